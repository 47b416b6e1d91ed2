"""GPU parity of the Metropolis path against the reference goldens and the
oracle, through the C ABI (bit-exact: configurations, energies, streams,
accept counts)."""
import zlib

import numpy as np
import pytest

import brawl_gb300 as B
from brawl_gb300 import inputs as I
from brawl_gb300 import metropolis as anneal
from brawl_gb300 import netcdf_io as NC
from brawl_gb300 import output as OUT
from oracle import oracle as O
from tests import golden_io as G

pytestmark = pytest.mark.gpu

RY_TO_EV = 13.605693122


def random_V(rng, ns, nsh, scale_ev=0.05):
    """Symmetric V_ex per shell, uniform[-scale, scale] eV, in Ry."""
    V = np.zeros((ns, ns, nsh))
    for sh in range(nsh):
        a = rng.uniform(-scale_ev, scale_ev, size=(ns, ns))
        V[:, :, sh] = np.triu(a) + np.triu(a, 1).T
    return V / RY_TO_EV


def equi_numbers(n_atoms, ns):
    base = np.full(ns, n_atoms // ns, dtype=np.int64)
    base[: n_atoms - base.sum()] += 1
    return base


def conc_vector(ns):
    c = np.zeros(ns + 1)
    c[1:] = 1.0 / ns
    return c


# ---------------------------------------------------------------------------
# goldens through the GPU
# ---------------------------------------------------------------------------
MET = [("01_serial_metropolis", 0)] + [("02_parallel_metropolis", r) for r in range(4)]


@pytest.mark.parametrize("test,rank", MET)
def test_golden_anneal_on_gpu(test, rank, tmp_path):
    p, V = G.load_inputs(test)
    m = I.read_metropolis_file(G.path(test, "metropolis.inp"))
    ch = B.Chain(B.Setup.from_run_params(p), V)
    seed = ch.f90_init_genrand(0, rank)
    assert seed == 110179 + 11 * rank
    ch.initial_setup(p.species_concentrations, p.numbers_or_none())
    out = anneal.simulated_annealing(ch, m, p.wc_range)
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
    assert np.array_equal(rho["U_data"], out["energies_of_T"])
    if test.startswith("02"):
        diag = OUT.diagnostics_lines(out["temperature"], out["energies_of_T"], out["C_of_T"],
                                     out["acceptance_of_T"])
        assert diag == G.text(test, tag + "_energy_diagnostics.dat")
    if test.startswith("02") and rank == 2:
        # the configuration file itself, byte for byte
        path = tmp_path / "init.nc"
        NC.write_config(str(path), out["initial_configs"][0], p)
        with open(G.path("netcdf", "02_proc_0002_initial_config_at_0300.0.nc"), "rb") as f:
            assert path.read_bytes() == f.read()


def test_golden_ensemble_in_one_batch():
    """The four MPI ranks of golden test 02 as the chains of one batch
    (simulated_annealing_ensemble): every rank's outputs are its golden
    files, and the ensemble average (comms_reduce_metropolis_results) is
    av_energy_diagnostics.dat and av_radial_density.nc."""
    test = "02_parallel_metropolis"
    p, V = G.load_inputs(test)
    m = I.read_metropolis_file(G.path(test, "metropolis.inp"))
    setup = B.Setup.from_run_params(p)
    chains = [dict(setup=setup, V=V, seed=110179 + 11 * r, beta=0.0, nbr_swap=m.nbr_swap,
                   species_concentrations=p.species_concentrations, species_numbers=p.numbers_or_none())
              for r in range(4)]
    res = anneal.simulated_annealing_ensemble(B.Batch(chains), m, p.wc_range)
    for r, out in enumerate(res["ranks"]):
        tag = "proc_%04d" % r
        assert np.array_equal(out["initial_configs"][0], G.config_zyx(test, tag + "_initial_config_at_0300.0.npz"))
        assert np.array_equal(out["final_configs"][0], G.config_zyx(test, tag + "_final_config_at_0300.0.npz"))
        lines = [OUT.energy_trajectory_header()] + [
            OUT.energy_trajectory_line(s, e) for s, e in zip(out["traj_step"], out["traj_energy"])]
        assert lines == G.text(test, tag + "_energy_trajectory_at_T_0300.0.dat")
        rho = G.npz(test, tag + "_rho_of_T.npz")
        assert np.array_equal(rho["rho_data"], out["rho_of_T"])
        diag = OUT.diagnostics_lines(out["temperature"], out["energies_of_T"], out["C_of_T"],
                                     out["acceptance_of_T"])
        assert diag == G.text(test, tag + "_energy_diagnostics.dat")
    av = res["average"]
    diag = OUT.diagnostics_lines(res["ranks"][0]["temperature"], av["energies_of_T"], av["C_of_T"],
                                 av["acceptance_of_T"])
    assert diag == G.text(test, "av_energy_diagnostics.dat")
    ref = G.npz(test, "av_radial_density.npz")
    assert np.array_equal(ref["rho_data"], av["rho_of_T"])
    assert np.array_equal(ref["U_data"], av["energies_of_T"])


# ---------------------------------------------------------------------------
# trial-level parity with the oracle
# ---------------------------------------------------------------------------
SYSTEMS = [
    # lattice, n, ns, nsh, T, trials, nbr_swap
    ("fcc", (4, 4, 4), 2, 2, 300.0, 60000, False),
    ("fcc", (3, 4, 5), 5, 6, 1500.0, 40000, False),
    ("bcc", (4, 4, 4), 4, 6, 100.0, 60000, False),
    ("bcc", (3, 5, 4), 3, 10, 800.0, 30000, False),
    ("bcc", (6, 6, 6), 4, 4, 3000.0, 40000, True),
    ("fcc", (2, 2, 2), 3, 6, 500.0, 20000, False),   # neighbours wrap more than once
    ("bcc", (1, 2, 1), 2, 10, 500.0, 5000, False),   # offsets reach the site itself
    ("simple_cubic", (3, 3, 3), 2, 2, 400.0, 20000, False),
    ("simple_cubic", (2, 3, 4), 3, 1, 50.0, 20000, True),
    ("fcc", (4, 4, 4), 4, 3, 5.0, 30000, False),     # nearly every uphill move rejected
    ("bcc", (3, 3, 4), 9, 8, 700.0, 20000, False),   # many species: no difference table
    ("fcc", (3, 3, 3), 15, 2, 2000.0, 20000, False),
]


def _oracle_run(lattice, n, V, seed, T, trials, nbr_swap, conc, nums):
    mod = O.OracleModel(lattice, *n, V)
    r = O.OracleRng(seed)
    cfg, conc2 = mod.initial_setup(r, conc, nums)
    beta = 1.0 / (T * B.K_B_IN_RY)
    acc, c = mod.mc_run(cfg, r, beta, trials, nbr_swap)
    return mod, cfg, r, acc, c, beta


@pytest.mark.parametrize("system", SYSTEMS, ids=lambda s: f"{s[0]}-{s[1]}-s{s[2]}-sh{s[3]}-T{s[4]}")
def test_metropolis_matches_oracle(system):
    lattice, n, ns, nsh, T, trials, nbr = system
    rng = np.random.default_rng(zlib.crc32(repr(system).encode()))
    V = random_V(rng, ns, nsh)
    setup = B.Setup(lattice, *n, ns, nsh)
    nums = equi_numbers(setup.n_atoms, ns)
    seed = int(rng.integers(1, 2**31))
    mod, cfg, r, acc, c, beta = _oracle_run(lattice, n, V, seed, T, trials, nbr, conc_vector(ns), nums)
    ch = B.Chain(setup, V)
    ch.seed(seed)
    ch.initial_setup(conc_vector(ns), nums)
    # split the run in uneven chunks: state must carry across calls
    acc_gpu = 0
    for chunk in (trials // 3, trials // 7, trials - trials // 3 - trials // 7):
        acc_gpu += ch.metropolis(beta, chunk, nbr)
    assert acc_gpu == acc
    assert np.array_equal(ch.config(), cfg)
    cnt = ch.counters()
    assert cnt["trials"] == c.trials and cnt["evaluated"] == c.evaluated
    assert cnt["accepted"] == c.accepted and cnt["exp_tests"] == c.exp_tests
    # the streams continue identically
    assert np.array_equal(ch.genrand(1500), np.array([r.uniform() for _ in range(1500)]))
    assert ch.total_energy() == mod.total_energy(cfg)


SPEC_SYSTEMS = [s for s in SYSTEMS if s[0] != "simple_cubic"]


@pytest.mark.parametrize("nc", [1, 2, 3, 4])
def test_speculative_rounds_match_oracle(nc):
    """Every fcc/bcc system (tiny lattices where most candidates conflict,
    nbr_swap, near-zero temperature, many species) in one batch, run with nc
    trials per speculative round, in uneven chunks: the oracle's trajectory,
    counters and streams, bit for bit."""
    chains, expect = [], []
    for system in SPEC_SYSTEMS:
        lattice, n, ns, nsh, T, trials, nbr = system
        rng = np.random.default_rng(zlib.crc32(repr(system).encode()))
        V = random_V(rng, ns, nsh)
        setup = B.Setup(lattice, *n, ns, nsh)
        nums = equi_numbers(setup.n_atoms, ns)
        seed = int(rng.integers(1, 2**31))
        mod, cfg, r, acc, c, beta = _oracle_run(lattice, n, V, seed, T, trials, nbr, conc_vector(ns), nums)
        chains.append(dict(setup=setup, V=V, seed=seed, beta=beta, nbr_swap=nbr,
                           species_concentrations=conc_vector(ns), species_numbers=nums))
        expect.append((trials, cfg, acc, c, r, mod))
    b = B.Batch(chains)
    b.set_speculation(nc)
    trials = np.array([e[0] for e in expect])
    acc = np.zeros(len(chains), dtype=np.int64)
    for frac in (3, 7):
        acc += b.metropolis(trials // frac)
    acc += b.metropolis(trials - trials // 3 - trials // 7)
    cnt = b.counters()
    names = B.COUNTER_NAMES
    for k, (t, cfg, a, c, r, mod) in enumerate(expect):
        assert acc[k] == a, SPEC_SYSTEMS[k]
        assert np.array_equal(b.config(k), cfg), SPEC_SYSTEMS[k]
        row = dict(zip(names, cnt[k]))
        assert row["evaluated"] == c.evaluated and row["exp_tests"] == c.exp_tests
        # the streams continue identically
        g = O.OracleRng(1)
        g.set_state_words(b.rng_state(k))
        assert [g.uniform() for _ in range(700)] == [r.uniform() for _ in range(700)]


def test_all_moves_on_the_exact_tier():
    """With every V equal, every swap's dE is exactly zero: each evaluated
    trial needs the FP64 reference-order sums (dE == 0 draws, exp(-0) = 1)."""
    setup = B.Setup("fcc", 3, 3, 3, 3, 3)
    V = np.full((3, 3, 3), 0.0123)
    nums = equi_numbers(setup.n_atoms, 3)
    mod, cfg, r, acc, c, beta = _oracle_run("fcc", (3, 3, 3), V, 99, 300.0, 5000, False,
                                            conc_vector(3), nums)
    ch = B.Chain(setup, V)
    ch.seed(99)
    ch.initial_setup(conc_vector(3), nums)
    assert ch.metropolis(beta, 5000) == acc
    assert np.array_equal(ch.config(), cfg)
    cnt = ch.counters()
    assert cnt["exact_path"] == cnt["evaluated"] > 0


def test_zero_interactions_and_infinite_beta():
    """V = 0: dE is +0 exactly, the move draws and exp(-beta*0) decides; at
    T = 0 beta is +inf and -inf*0 is NaN, so every such move is rejected."""
    setup = B.Setup("bcc", 3, 3, 3, 2, 2)
    V = np.zeros((2, 2, 2))
    nums = equi_numbers(setup.n_atoms, 2)
    for beta in (1000.0, float("inf")):
        mod = O.OracleModel("bcc", 3, 3, 3, V)
        r = O.OracleRng(7)
        cfg, _ = mod.initial_setup(r, conc_vector(2), nums)
        acc, c = mod.mc_run(cfg, r, beta, 3000)
        ch = B.Chain(setup, V)
        ch.seed(7)
        ch.initial_setup(conc_vector(2), nums)
        assert ch.metropolis(beta, 3000) == acc
        assert np.array_equal(ch.config(), cfg)


def test_batch_equals_individual_and_serial():
    """Chains of different lattices, sizes, species and shells run together
    in one launch give exactly what each gives alone (and what the oracle
    gives); the one-chain-per-launch path gives the same."""
    rng = np.random.default_rng(5)
    specs = [("bcc", (4, 4, 4), 4, 6), ("fcc", (3, 3, 3), 2, 2), ("bcc", (6, 5, 4), 3, 10),
             ("fcc", (5, 5, 5), 5, 3), ("simple_cubic", (3, 3, 3), 2, 2), ("bcc", (2, 2, 2), 4, 5)]
    chains, expect = [], []
    for k, (lat, n, ns, nsh) in enumerate(specs):
        V = random_V(rng, ns, nsh)
        T = float(rng.uniform(100, 3000))
        setup = B.Setup(lat, *n, ns, nsh)
        nums = equi_numbers(setup.n_atoms, ns)
        seed = 110179 + 11 * k
        beta = 1.0 / (T * B.K_B_IN_RY)
        chains.append(dict(setup=setup, V=V, seed=seed, beta=beta,
                           species_concentrations=conc_vector(ns), species_numbers=nums))
        trials = 7 * setup.n_atoms
        mod, cfg, r, acc, c, _ = _oracle_run(lat, n, V, seed, T, trials, False, conc_vector(ns), nums)
        expect.append((trials, cfg, acc, mod.total_energy(cfg)))
    trials = np.array([e[0] for e in expect])
    b = B.Batch(chains)
    acc = b.metropolis(trials)
    energies = b.total_energy()
    b2 = B.Batch(chains)
    acc2 = b2.metropolis_serial(trials)
    for k, (t, cfg, a, e) in enumerate(expect):
        assert acc[k] == a and acc2[k] == a
        assert np.array_equal(b.config(k), cfg) and np.array_equal(b2.config(k), cfg)
        assert energies[k] == e


def test_batched_replica_shape_matches_oracle():
    """The batched-replica workload's shape in small: bcc chains of several
    sizes, 4 species, 6 shells (every lane entry a neighbour), log-spaced
    temperatures, seeds 110179 + 11 r, in one launch; each chain equals the
    oracle."""
    rng = np.random.default_rng(64)
    V = random_V(rng, 4, 6)
    Ls = [3, 4, 5, 4, 6, 3, 5, 7]
    chains, expect = [], []
    for r, L in enumerate(Ls):
        T = 100.0 * 30.0 ** (r / (len(Ls) - 1))
        setup = B.Setup("bcc", L, L, L, 4, 6)
        seed = 110179 + 11 * r
        chains.append(dict(setup=setup, V=V, seed=seed, beta=1.0 / (T * B.K_B_IN_RY),
                           species_concentrations=conc_vector(4)))
        trials = 10 * setup.n_atoms
        mod, cfg, r_, acc, c, _ = _oracle_run("bcc", (L, L, L), V, seed, T, trials, False,
                                              conc_vector(4), None)
        expect.append((trials, cfg, acc, c))
    b = B.Batch(chains)
    acc = b.metropolis(np.array([e[0] for e in expect]))
    cnt = b.counters()
    for k, (t, cfg, a, c) in enumerate(expect):
        assert acc[k] == a, Ls[k]
        assert np.array_equal(b.config(k), cfg), Ls[k]
        row = dict(zip(B.COUNTER_NAMES, cnt[k]))
        # exp_tests is counted from the words the kernel consumed
        assert row["evaluated"] == c.evaluated and row["exp_tests"] == c.exp_tests


def test_metropolis_from_host_buffers():
    """brawl_batch_metropolis_host (pinned buffers used in place, pageable
    ones through a copy) gives what set_configs + metropolis + get_configs
    give; a bad species flags its chain, which runs no trial, and the call
    fails."""
    import torch
    rng = np.random.default_rng(12)
    V = random_V(rng, 3, 4)
    Ls = [3, 5, 4, 6]
    def make():
        return B.Batch([dict(setup=B.Setup("bcc", L, L, L, 3, 4), V=V, seed=7 + r,
                             beta=1.0 / (600.0 * B.K_B_IN_RY), species_concentrations=conc_vector(3))
                        for r, L in enumerate(Ls)])
    a, b, c = make(), make(), make()
    trials = np.array([10 * 2 * L ** 3 for L in Ls], dtype=np.int64)
    grids = a.get_configs()
    pinned = torch.empty(a.grid_bytes, dtype=torch.int8, pin_memory=True).numpy()
    pinned[:] = grids
    pageable = grids.copy()
    for _ in range(3):
        acc_a = a.metropolis_host(pinned, trials)
        acc_c = c.metropolis_host(pageable, trials)
        b.set_configs(b.get_configs())
        acc_b = b.metropolis(trials)
        ref = b.get_configs()
        assert list(acc_a) == list(acc_b) == list(acc_c)
        assert np.array_equal(pinned, ref) and np.array_equal(pageable, ref)
    bad = pinned.copy()
    occupied = np.nonzero(bad)[0]
    bad[occupied[0]] = 9                       # species 9 of 3, in chain 0's grid
    with pytest.raises(B.BrawlError):
        a.metropolis_host(bad, trials)
    cnt = a.counters()
    assert cnt[0][0] == 3 * trials[0]          # chain 0 ran no trial in the failed call
    assert cnt[1][0] == 4 * trials[1]          # the others did


def test_initial_setup_modes_match_oracle():
    rng = np.random.default_rng(11)
    for lat, n, ns in (("fcc", (4, 3, 2), 5), ("bcc", (5, 5, 5), 3), ("simple_cubic", (2, 2, 3), 4)):
        setup = B.Setup(lat, *n, ns, 1)
        V = random_V(rng, ns, 1)
        conc = np.zeros(ns + 1)
        conc[1:] = rng.dirichlet(np.ones(ns))
        for nums in (None, equi_numbers(setup.n_atoms, ns)):
            mod = O.OracleModel(lat, *n, V)
            r = O.OracleRng(1234)
            cfg, conc_o = mod.initial_setup(r, conc, nums)
            ch = B.Chain(setup, V)
            ch.seed(1234)
            conc_g = ch.initial_setup(conc, nums)
            assert np.array_equal(ch.config(), cfg)
            assert np.array_equal(conc_g, conc_o)
            assert np.array_equal(ch.genrand(10), np.array([r.uniform() for _ in range(10)]))


def test_energies_match_oracle():
    rng = np.random.default_rng(3)
    for lat, n, ns, nsh in (("bcc", (5, 4, 3), 4, 10), ("fcc", (4, 4, 4), 5, 6),
                            ("simple_cubic", (3, 4, 2), 3, 2)):
        V = random_V(rng, ns, nsh)
        setup = B.Setup(lat, *n, ns, nsh)
        mod = O.OracleModel(lat, *n, V)
        r = O.OracleRng(42)
        cfg, _ = mod.initial_setup(r, conc_vector(ns), equi_numbers(setup.n_atoms, ns))
        ch = B.Chain(setup, V)
        ch.set_config(cfg)
        assert ch.total_energy() == mod.total_energy(cfg)
        occ = np.argwhere(cfg != 0)[:20]
        for z, y, x in occ:
            idx = (1, x + 1, y + 1, z + 1)
            assert ch.site_energy(idx) == mod.site_energy(cfg, x, y, z)
        (z1, y1, x1), (z2, y2, x2) = occ[0], occ[-1]
        assert ch.pair_energy((1, x1 + 1, y1 + 1, z1 + 1), (1, x2 + 1, y2 + 1, z2 + 1)) == \
            mod.pair_energy(cfg, (x1, y1, z1), (x2, y2, z2))


@pytest.mark.parametrize("lat,n,ns,wc", [("fcc", (4, 4, 4), 5, 3), ("bcc", (4, 4, 4), 4, 2),
                                         ("bcc", (6, 7, 8), 3, 6), ("fcc", (2, 3, 2), 2, 8),
                                         ("simple_cubic", (3, 3, 3), 2, 4),
                                         ("bcc", (12, 12, 12), 4, 3)])
def test_radial_densities_match_oracle(lat, n, ns, wc):
    rng = np.random.default_rng(17)
    V = random_V(rng, ns, 1)
    setup = B.Setup(lat, *n, ns, 1)
    mod = O.OracleModel(lat, *n, V)
    r = O.OracleRng(77)
    cfg, _ = mod.initial_setup(r, conc_vector(ns), equi_numbers(setup.n_atoms, ns))
    shells = mod.lattice_shells(cfg, wc)
    rho_o, _ = mod.radial_densities(cfg, shells)
    ch = B.Chain(setup, V)
    ch.set_config(cfg)
    assert np.array_equal(ch.lattice_shells(wc), shells)
    rho_g = ch.radial_densities(shells)
    assert np.array_equal(rho_g, rho_o)


def test_rng_interface_matches_reference_generator():
    setup = B.Setup("fcc", 2, 2, 2, 2, 1)
    ch = B.Chain(setup, np.zeros((2, 2, 1)))
    for seed in (110179, 5489, 1, 4294967295):
        ch.seed(seed)
        r = O.OracleRng(seed)
        assert np.array_equal(ch.genrand(2000), np.array([r.uniform() for _ in range(2000)]))
    st = ch.rng_state()
    ch.set_rng_state(st)
    assert st[624] <= 624


def test_invalid_inputs_return_status():
    with pytest.raises(B.BrawlError) as e:
        B.Chain(B.Setup("fcc", 2, 2, 2, 2, 7), np.zeros((2, 2, 7)))
    assert e.value.code == 1
    with pytest.raises(B.BrawlError):
        B.Chain(B.Setup("bcc", 2, 2, 2, 2, 11), np.zeros((2, 2, 11)))
    ch = B.Chain(B.Setup("fcc", 2, 2, 2, 2, 1), np.zeros((2, 2, 1)))
    bad = np.zeros(ch.setup.grid_shape, dtype=np.int8)
    with pytest.raises(B.BrawlError):
        ch.set_config(bad)          # occupied sites must hold a species
    with pytest.raises(B.BrawlError):
        ch.initial_setup(np.array([0.0, 0.0, 0.0]))   # counts cannot reach n_atoms


@pytest.mark.parametrize("nbr_swap", [False, True])
def test_decorrelated_samples_match_oracle(nbr_swap):
    """metropolis_decorrelated_samples through the C ABI against the
    reference's loop on the oracle, trial by trial: burn-in acceptances,
    sampled energies, acceptances and configurations, final stream."""
    from tests.test_drivers_cpu import reference_loop, small_system
    m = I.MetropolisParams(mode="decorrelated_samples", n_mc_steps=5000, n_sample_steps=700,
                           burn_in=True, n_burn_in_steps=400, T=1500.0, T_steps=4, delta_T=-300.0,
                           nbr_swap=nbr_swap)
    mod, cfg, r, V = small_system(11)
    ch = B.Chain(B.Setup("bcc", 3, 3, 3, 3, 2), V)
    ch.set_config(cfg)
    ch.set_rng_state(r.state_words())
    burn, steps, energies, accs, cfgs = reference_loop(mod, cfg, r, m)
    out = anneal.decorrelated_samples(ch, m)
    assert list(out["burn_in_accepted"]) == burn
    assert list(out["sample_step"]) == steps
    assert list(out["sample_energy"]) == energies
    assert list(out["sample_accepted"]) == accs
    assert all(np.array_equal(a, b) for a, b in zip(out["configs"], cfgs))
    g = O.OracleRng(1)
    g.set_state_words(ch.rng_state())
    assert [g.uniform() for _ in range(700)] == [r.uniform() for _ in range(700)]


def test_annealing_alro_matches_oracle():
    """The annealing driver's ALRO (store_state accumulated on the device)
    against the reference's loop on the oracle, bit for bit."""
    from tests.test_drivers_cpu import reference_alro, small_system
    m = I.MetropolisParams(mode="simulated_annealing", n_mc_steps=2700, n_sample_steps=54,
                           calculate_energies=True, calculate_asro=False, n_sample_steps_asro=54,
                           calculate_alro=True, n_sample_steps_alro=162, n_sample_steps_trajectory=54,
                           T=1200.0, T_steps=4, delta_T=-250.0)
    mod, cfg, r, V = small_system(23)
    ch = B.Chain(B.Setup("bcc", 3, 3, 3, 3, 2), V)
    ch.set_config(cfg)
    ch.set_rng_state(r.state_words())
    ref = reference_alro(mod, cfg.copy(), r, m)
    out = anneal.simulated_annealing(ch, m, 2, record_configs=False)
    assert np.array_equal(out["order_of_T"], ref)


def test_largest_lattices_match_oracle():
    """Maximum sizes in one batch: the batched workload's largest chain (bcc
    L = 24, 27648 sites, 4 species, 6 shells: the shared-memory halo kernel
    with every lane entry a neighbour) and an fcc L = 40 chain (256000
    sites, 3 species, 3 shells), whose lattice exceeds shared memory and
    stays in HBM; one sweep each, and each equals the oracle: accepts,
    configuration, counters, energy and the stream's continuation."""
    rng = np.random.default_rng(2424)
    cases = [("bcc", 24, 4, 6, 600.0), ("fcc", 40, 3, 3, 900.0)]
    chains, expect = [], []
    for k, (lat, L, ns, nsh, T) in enumerate(cases):
        V = random_V(rng, ns, nsh)
        setup = B.Setup(lat, L, L, L, ns, nsh)
        seed = 110179 + 11 * k
        chains.append(dict(setup=setup, V=V, seed=seed, beta=1.0 / (T * B.K_B_IN_RY),
                           species_concentrations=conc_vector(ns)))
        trials = setup.n_atoms
        expect.append((trials,) + _oracle_run(lat, (L, L, L), V, seed, T, trials, False, conc_vector(ns), None))
    b = B.Batch(chains)
    acc = b.metropolis(np.array([e[0] for e in expect]))
    cnt = b.counters()
    E = b.total_energy()
    for k, (trials, mod, cfg, r, a, c, _) in enumerate(expect):
        assert acc[k] == a, cases[k]
        assert np.array_equal(b.config(k), cfg), cases[k]
        row = dict(zip(B.COUNTER_NAMES, cnt[k]))
        assert row["trials"] == c.trials and row["evaluated"] == c.evaluated
        assert row["accepted"] == c.accepted and row["exp_tests"] == c.exp_tests
        assert E[k] == mod.total_energy(cfg), cases[k]
        cont = O.OracleRng(1)
        cont.set_state_words(b.rng_state(k))
        assert [cont.uniform() for _ in range(200)] == [r.uniform() for _ in range(200)]


def test_autotune_keeps_the_state_and_the_trajectories():
    """brawl_batch_autotune times every trials-per-round depth from one
    state and restores it after each: configurations, streams and counters
    are unchanged by the call, and the runs after it still equal the
    oracle's whatever depth it kept."""
    rng = np.random.default_rng(65)
    V = random_V(rng, 4, 6)
    Ls = [4, 6, 3, 5]
    chains, expect = [], []
    for r, L in enumerate(Ls):
        T = 200.0 * 5.0 ** (r / (len(Ls) - 1))
        setup = B.Setup("bcc", L, L, L, 4, 6)
        seed = 110179 + 11 * r
        chains.append(dict(setup=setup, V=V, seed=seed, beta=1.0 / (T * B.K_B_IN_RY),
                           species_concentrations=conc_vector(4)))
        trials = 6 * setup.n_atoms
        mod, cfg, r_, acc, c, _ = _oracle_run("bcc", (L, L, L), V, seed, T, trials, False, conc_vector(4), None)
        expect.append((trials, cfg, acc, c))
    b = B.Batch(chains)
    before = ([b.config(k) for k in range(len(Ls))], [b.rng_state(k) for k in range(len(Ls))], b.counters())
    depth, ms = b.autotune(np.array([3 * e[0] for e in expect]))
    assert 1 <= depth <= 4 and ms.shape == (4,) and (ms > 0).all()
    assert ms[depth - 1] == ms.min()
    for k in range(len(Ls)):
        assert np.array_equal(b.config(k), before[0][k])
        assert np.array_equal(b.rng_state(k), before[1][k])
    assert np.array_equal(b.counters(), before[2])
    acc = b.metropolis(np.array([e[0] for e in expect]))
    for k, (t, cfg, a, c) in enumerate(expect):
        assert acc[k] == a and np.array_equal(b.config(k), cfg), Ls[k]


def test_classes_run_their_own_depths_and_autotune_keeps_state():
    """Shared-memory chains in classes (lattice, L, species, shells), each
    class in its own launch: with different trials per round per class the
    runs equal the oracle's; brawl_batch_autotune_classes leaves the state
    as it found it and reports a depth per class."""
    rng = np.random.default_rng(66)
    V = random_V(rng, 4, 6)
    Ls = [4, 6, 4, 6, 5]
    chains, expect = [], []
    for r, L in enumerate(Ls):
        T = 300.0 * 4.0 ** (r / (len(Ls) - 1))
        setup = B.Setup("bcc", L, L, L, 4, 6)
        seed = 110179 + 11 * r
        chains.append(dict(setup=setup, V=V, seed=seed, beta=1.0 / (T * B.K_B_IN_RY),
                           species_concentrations=conc_vector(4)))
        trials = 5 * setup.n_atoms
        mod, cfg, r_, acc, c, _ = _oracle_run("bcc", (L, L, L), V, seed, T, trials, False, conc_vector(4), None)
        expect.append((trials, cfg, acc, c))
    b = B.Batch(chains)
    cls = b.chain_classes()
    assert cls[0] == cls[2] and cls[1] == cls[3] and len(set(cls.tolist())) == 3
    before = ([b.config(k) for k in range(len(Ls))], [b.rng_state(k) for k in range(len(Ls))], b.counters())
    tuned = b.autotune_classes(np.array([2 * e[0] for e in expect]))
    assert len(tuned["classes"]) == 3
    assert all(1 <= c["trials_per_round"] <= 4 for c in tuned["classes"])
    for k in range(len(Ls)):
        assert np.array_equal(b.config(k), before[0][k])
        assert np.array_equal(b.rng_state(k), before[1][k])
    assert np.array_equal(b.counters(), before[2])
    b.set_class_depths([3, 1, 2])
    half = [e[0] // 2 for e in expect]
    acc1 = b.metropolis(np.array(half))
    b.set_class_depths([1, 4, 1])
    acc2 = b.metropolis(np.array([e[0] - h for e, h in zip(expect, half)]))
    for k, (t, cfg, a, c) in enumerate(expect):
        assert acc1[k] + acc2[k] == a and np.array_equal(b.config(k), cfg), Ls[k]


def test_anneal_sweeps_equal_per_sweep_calls():
    """brawl_anneal_sweeps / brawl_batch_anneal_sweeps (sweeps back to back,
    each sweep's energy taken from a snapshot on another stream) give the
    energies, accepted counts, configurations and streams of one
    metropolis call + one total_energy call per sweep; with accumulate the
    sampling sums are brawl_batch_energy_sample's."""
    rng = np.random.default_rng(71)
    V = random_V(rng, 2, 2)
    setup = B.Setup("fcc", 4, 4, 4, 2, 2)
    beta = 1.0 / (700.0 * B.K_B_IN_RY)
    a, b_ = B.Chain(setup, V), B.Chain(setup, V)
    for ch in (a, b_):
        ch.seed(4242)
        ch.initial_setup(conc_vector(2), equi_numbers(setup.n_atoms, 2))
    sweep = setup.n_atoms
    E_ref, acc_ref = [], 0
    for _ in range(9):
        acc_ref += a.metropolis(beta, sweep)
        E_ref.append(a.total_energy())
    E, acc = b_.anneal_sweeps(beta, 9, sweep)
    assert acc == acc_ref and np.array_equal(E, np.array(E_ref))
    assert np.array_equal(a.config(), b_.config()) and np.array_equal(a.rng_state(), b_.rng_state())
    E0, acc0 = b_.anneal_sweeps(beta, 3, sweep, energies=False)
    acc_ref = sum(a.metropolis(beta, sweep) for _ in range(3))
    assert E0 is None and acc0 == acc_ref and np.array_equal(a.config(), b_.config())
    # neighbour swaps (monte_carlo_step_nbr)
    E_ref, acc_ref = [], 0
    for _ in range(4):
        acc_ref += a.metropolis(beta, sweep, nbr_swap=True)
        E_ref.append(a.total_energy())
    E, acc = b_.anneal_sweeps(beta, 4, sweep, nbr_swap=True)
    assert acc == acc_ref and np.array_equal(E, np.array(E_ref))
    assert np.array_equal(a.config(), b_.config()) and np.array_equal(a.rng_state(), b_.rng_state())

    # a batch of two classes (different L) with their own betas, sums on the device
    V4 = random_V(rng, 4, 6)
    chains = []
    for r, L in enumerate([4, 5, 4]):
        chains.append(dict(setup=B.Setup("bcc", L, L, L, 4, 6), V=V4, seed=110179 + 11 * r,
                           beta=1.0 / ((400.0 + 300.0 * r) * B.K_B_IN_RY), species_concentrations=conc_vector(4)))
    p2, q2 = B.Batch(chains), B.Batch(chains)
    q2.set_class_depths([2, 1])  # per-class launches, the L = 4 class two trials per round
    n = min(c["setup"].n_atoms for c in chains)
    for x in (p2, q2):
        x.sampling_reset(0)
    E_ref, acc_ref = [], np.zeros(3, dtype=np.int64)
    for _ in range(6):
        acc_ref += p2.metropolis(np.full(3, n))
        E_ref.append(p2.energy_sample())
    E, acc = q2.anneal_sweeps(6, n, accumulate=True)
    assert np.array_equal(E, np.array(E_ref)) and np.array_equal(acc, acc_ref)
    for k in range(3):
        assert np.array_equal(p2.config(k), q2.config(k))
    s_p = p2.temperature_stats(6, 6 * n, 500.0, 500.0 * B.K_B_IN_RY, True)
    s_q = q2.temperature_stats(6, 6 * n, 500.0, 500.0 * B.K_B_IN_RY, True)
    assert np.array_equal(s_p[0], s_q[0]) and np.array_equal(s_p[1], s_q[1])


def _temper(y):
    y ^= y >> 11
    y ^= (y << 7) & 0x9D2C5680
    y ^= (y << 15) & 0xEFC60000
    y ^= y >> 18
    return y & 0xFFFFFFFF


def _untemper(y):
    """The mt19937 state word whose tempered output is y."""
    y ^= y >> 18
    y ^= (y << 15) & 0xEFC60000
    t = y
    for _ in range(5):
        t = y ^ ((t << 7) & 0x9D2C5680)
    y = t & 0xFFFFFFFF
    t = y
    for _ in range(3):
        t = y ^ (t >> 11)
    return t & 0xFFFFFFFF


def test_initial_setup_on_interval_boundaries():
    """A stream word on the boundary of two species' intervals: every species
    whose quota is open takes the site in turn and uses up one of its quota
    (src/initialise.F90's loop over l), the last one keeping it.  With one
    side already full the word is an ordinary draw (device equals the
    oracle, word for word); with both open a quota is used up twice, the
    configuration can never be completed (the reference loops forever) and
    the device reports the chain at its draw limit."""
    for x in (0, 1, 0x80000000, 0x12345678, 0xFFFFFFFF):
        assert _temper(_untemper(x)) == x
    rng = np.random.default_rng(17)
    setup = B.Setup("fcc", 2, 2, 2, 2, 1)  # 32 sites
    V = random_V(rng, 2, 1)
    base = O.OracleRng(4321).state_words()
    # species 1 holds [0, 2^27], species 2 [2^27, 2^32 - 1] (1 : 31 atoms)
    nums = np.array([1, 31], dtype=np.int64)
    st = base.copy()
    st[0] = _untemper(100)            # species 1: its only atom
    st[1] = _untemper(1 << 27)        # the boundary, species 1 already full
    st[624] = 0
    mod = O.OracleModel("fcc", 2, 2, 2, V)
    r = O.OracleRng(1)
    r.set_state_words(st)
    cfg, conc_o = mod.initial_setup(r, np.array([0.0, 0.5, 0.5]), nums)
    ch = B.Chain(setup, V)
    ch.set_rng_state(st)
    conc_g = ch.initial_setup(np.array([0.0, 0.5, 0.5]), nums)
    assert np.array_equal(ch.config(), cfg) and np.array_equal(conc_g, conc_o)
    assert np.array_equal(ch.genrand(8), np.array([r.uniform() for _ in range(8)]))
    # both quotas open at the boundary word (16 : 16, boundary 2^31), drawn
    # first or in the middle of a 32-word batch
    for at in (0, 5):
        st = base.copy()
        st[at] = _untemper(1 << 31)
        st[624] = 0
        ch = B.Chain(setup, V)
        ch.set_rng_state(st)
        with pytest.raises(B.BrawlError):
            ch.initial_setup(np.array([0.0, 0.5, 0.5]), np.array([16, 16], dtype=np.int64))
