"""Host logic of the Metropolis drivers without a GPU: the drivers run over
a chain backed by the oracle, and must make the calls the reference's loops
imply (src/metropolis.F90:560-738 for decorrelated_samples), checked
against a trial-by-trial restatement of that loop."""
from __future__ import annotations

import numpy as np

import brawl_gb300 as B
from brawl_gb300 import inputs as I
from brawl_gb300 import metropolis as M
from oracle import oracle as O


class OracleChain:
    """The chain interface the drivers use, over the oracle."""

    def __init__(self, mod, cfg, rng, setup=None):
        self.mod, self.cfg, self.rng = mod, cfg, rng
        self.setup = setup

    def metropolis(self, beta, n_trials, nbr_swap=False):
        acc, _ = self.mod.mc_run(self.cfg, self.rng, beta, n_trials, nbr_swap)
        return acc

    def total_energy(self):
        return self.mod.total_energy(self.cfg)

    def anneal_sweeps(self, beta, n_sweeps, sweep_trials, nbr_swap=False, energies=True):
        E = np.zeros(n_sweeps) if energies else None
        acc = 0
        for i in range(n_sweeps):
            acc += self.metropolis(beta, sweep_trials, nbr_swap)
            if energies:
                E[i] = self.total_energy()
        return E, acc

    def config(self):
        return self.cfg.copy()

    def lattice_shells(self, wc_range):
        return self.mod.lattice_shells(self.cfg, wc_range)

    def radial_densities(self, shells):
        return self.mod.radial_densities(self.cfg, shells)[0]

    # ALRO on the host: store_state's +1.0 per occupied site and species
    def alro_reset(self):
        self._order = np.zeros(self.cfg.shape + (1, self.mod.ns))

    def alro_add(self):
        for s in range(1, self.mod.ns + 1):
            self._order[..., 0, s - 1] += (self.cfg == s)

    def alro(self):
        return self._order.copy()


def small_system(seed):
    rng = np.random.default_rng(seed)
    V = np.zeros((3, 3, 2))
    for sh in range(2):
        a = rng.uniform(-0.05, 0.05, size=(3, 3))
        V[:, :, sh] = (np.triu(a) + np.triu(a, 1).T) / 13.605693122
    mod = O.OracleModel("bcc", 3, 3, 3, V)
    r = O.OracleRng(seed)
    conc = np.array([0.0, 1 / 3, 1 / 3, 1 / 3])
    cfg, _ = mod.initial_setup(r, conc, np.array([18, 18, 18]))
    return mod, cfg, r, V


def reference_loop(mod, cfg, rng, m):
    """metropolis_decorrelated_samples, one trial at a time."""
    beta = None
    burn = []
    for j in range(m.T_steps):
        temp = m.T + float(j) * m.delta_T
        beta = 1.0 / (temp * B.K_B_IN_RY)
        acc = 0
        if m.burn_in:
            for _ in range(m.n_burn_in_steps):
                acc += mod.mc_run(cfg, rng, beta, 1, m.nbr_swap)[0]
        burn.append(acc)
    steps, energies, accs, cfgs = [], [], [], []
    acc = 0
    for i in range(1, m.n_mc_steps + 1):
        acc += mod.mc_run(cfg, rng, beta, 1, m.nbr_swap)[0]
        if i % m.n_sample_steps == 0:
            steps.append(i)
            energies.append(mod.total_energy(cfg))
            accs.append(acc)
            cfgs.append(cfg.copy())
            acc = 0
    return burn, steps, energies, accs, cfgs


def test_decorrelated_samples_host_logic():
    m = I.MetropolisParams(mode="decorrelated_samples", n_mc_steps=2300, n_sample_steps=300,
                           burn_in=True, n_burn_in_steps=150, T=1200.0, T_steps=3, delta_T=-400.0)
    mod, cfg, r, _ = small_system(7)
    # the same start for both: copy the configuration and the stream
    cfg_a, cfg_b = cfg.copy(), cfg.copy()
    ra, rb = O.OracleRng(1), O.OracleRng(1)
    ra.set_state_words(r.state_words())
    rb.set_state_words(r.state_words())
    burn, steps, energies, accs, cfgs = reference_loop(mod, cfg_a, ra, m)
    out = M.decorrelated_samples(OracleChain(mod, cfg_b, rb), m)
    assert list(out["burn_in_accepted"]) == burn
    assert list(out["sample_step"]) == steps == [300 * k for k in range(1, 8)]
    assert list(out["sample_energy"]) == energies
    assert list(out["sample_accepted"]) == accs
    assert all(np.array_equal(a, b) for a, b in zip(out["configs"], cfgs))
    assert np.array_equal(cfg_a, cfg_b)  # the 200 trials after the last sample ran too
    assert np.array_equal(ra.state_words(), rb.state_words())


class FakeRadialWalkers:
    """The radial interface save_rho_E uses, over fixed arrays."""

    def __init__(self, records, rhos):
        self.records, self.rhos, self.n = records, rhos, len(records)
        self.done = None

    def radial(self, w):
        return self.records[w].copy(), self.rhos[w].copy(), 0

    def radial_set_done(self, done):
        self.done = np.asarray(done, dtype=bool).copy()


def test_save_rho_E_bookkeeping():
    """save_rho_E (src/wang-landau.F90:359-396): bins complete when the
    walkers' summed radial_record reaches radial_samples; rho_saved (and the
    averaged rho_of_E) only once every bin is complete."""
    from brawl_gb300.wang_landau import save_rho_E
    rng = np.random.default_rng(3)
    bins, wc, ns = 6, 2, 3
    recs = [np.array([2, 0, 3, 1, 2, 2], dtype=np.int32), np.array([1, 2, 0, 2, 1, 2], dtype=np.int32)]
    rhos = [rng.uniform(0, 1, (bins, wc, ns, ns)) for _ in recs]
    W = FakeRadialWalkers(recs, rhos)
    st = {"rho_saved": False, "rho_of_E": None, "radial_min": 0.0}
    save_rho_E(W, 3, st)
    assert list(W.done) == [True, False, True, True, True, True]
    assert not st["rho_saved"] and st["rho_of_E"] is None
    assert st["radial_min"] == float(np.float32(5) / np.float32(6))
    W.records[0][1] = 1
    save_rho_E(W, 3, st)
    assert W.done.all() and st["rho_saved"]
    total = (W.records[0] + W.records[1]).astype(np.float64)
    assert np.array_equal(st["rho_of_E"], (rhos[0] + rhos[1]) / total[:, None, None, None])
    W.done = None
    save_rho_E(W, 3, st)                 # rho_saved: nothing more happens
    assert W.done is None


def reference_alro(mod, cfg, rng, m):
    """metropolis_simulated_annealing's ALRO (src/metropolis.F90:192-197,
    394-399, 444-447) on the oracle: per temperature the order array is
    zeroed, every n_sample_steps_alro trials store_state adds the
    occupancies, and order_of_T = order / real(n_save_alro)."""
    n_sweeps = m.n_mc_steps // m.n_sample_steps
    n_sweep_steps = m.n_mc_steps // n_sweeps
    n_save = int(np.floor(np.float32(m.n_mc_steps) / np.float32(m.n_sample_steps_alro)))
    out = []
    for j in range(m.T_steps):
        temp = m.T + float(j) * m.delta_T
        beta = 1.0 / (temp * B.K_B_IN_RY)
        order = np.zeros(cfg.shape + (1, mod.ns))
        for i in range(1, n_sweeps + 1):
            mod.mc_run(cfg, rng, beta, n_sweep_steps, m.nbr_swap)
            if (i * n_sweep_steps) % m.n_sample_steps_alro == 0:
                for s in range(1, mod.ns + 1):
                    order[..., 0, s - 1] += (cfg == s)
        out.append(order / float(np.float32(n_save)))
    return np.array(out)


def test_annealing_alro_host_logic():
    m = I.MetropolisParams(mode="simulated_annealing", n_mc_steps=540, n_sample_steps=54,
                           calculate_energies=True, calculate_asro=False, n_sample_steps_asro=54,
                           calculate_alro=True, n_sample_steps_alro=108, n_sample_steps_trajectory=54,
                           T=900.0, T_steps=3, delta_T=-300.0)
    mod, cfg, r, _ = small_system(21)
    ra, rb = O.OracleRng(1), O.OracleRng(1)
    ra.set_state_words(r.state_words())
    rb.set_state_words(r.state_words())
    ref = reference_alro(mod, cfg.copy(), ra, m)
    setup = B.Setup("bcc", 3, 3, 3, 3, 2)
    out = M.simulated_annealing(OracleChain(mod, cfg.copy(), rb, setup), m, 2, record_configs=False)
    assert out["order_of_T"].shape == ref.shape
    assert np.array_equal(out["order_of_T"], ref)
    assert np.allclose(out["order_of_T"].sum(axis=-1)[:, cfg > 0], 1.0)  # occupied sites: one species each


def test_compute_mean_energy():
    """compute_mean_energy (src/wang-landau.F90:457-477): beta per row, the
    canonical mean over the bin centres, low T at the low-energy end."""
    from brawl_gb300.wang_landau import compute_mean_energy
    bins = 50
    edges = -1.0 + np.arange(bins + 1) * 0.02
    lng = 40.0 * np.sin(np.linspace(0, np.pi, bins))      # a smooth ln g, largest mid-range
    me = compute_mean_energy(lng, edges, bins, 0.02)
    assert me.shape == (300, 2)
    assert np.allclose(me[:, 1], 1.0 / (B.K_B_IN_RY * np.arange(1, 301) * 10.0), rtol=0, atol=0)
    centres = edges[:bins] + 0.01
    assert np.all(me[:, 0] >= centres[0] - 1e-12) and np.all(me[:, 0] <= centres[-1] + 1e-12)
    assert me[0, 0] < me[-1, 0]                              # colder: lower mean energy


# ---------------------------------------------------------------------------
# Wang-Landau window optimisation and the configuration store's host side
# (src/wang-landau.F90:1211-1328, 1541-1615, 1686-1703)
# ---------------------------------------------------------------------------
from brawl_gb300 import wang_landau as WLD  # noqa: E402

QUARTERS = [[1, 128], [129, 256], [257, 384], [385, 512]]


def test_window_optimise_hand_cases():
    """Each case worked by hand from the reference's formulas: weights
    1/(steps/ABS(first-last+1)) normalised, mixed with the previous
    fractions by alpha, floored at 0.02, NINT(bins * frac), rounding settled
    on the windows by descending size."""
    # iteration 0: alpha = 1, fractions (1, 1/2, 1, 1/4) / 2.75 -> 186, 93, 186, 47
    iv, prev = WLD.window_optimise(0, QUARTERS, [1e6, 2e6, 1e6, 4e6], [0.25] * 4, 512)
    assert iv == [[1, 186], [187, 279], [280, 465], [466, 512]]
    assert np.allclose(prev, np.array([1.0, 0.5, 1.0, 0.25]) / 2.75, rtol=0, atol=1e-15)
    # iteration 2: alpha = 0.8 * 0.8 = 0.64 mixed with the previous fractions:
    # 137.59, 96.44, 174.45, 103.52 -> 138, 96, 174, 104
    iv, _ = WLD.window_optimise(2, QUARTERS, [1e6, 2e6, 1e6, 4e6], [0.1, 0.2, 0.3, 0.4], 512)
    assert iv == [[1, 138], [139, 234], [235, 408], [409, 512]]
    # equal work keeps equal windows
    iv, _ = WLD.window_optimise(1, QUARTERS, [1e6] * 4, [0.25] * 4, 512)
    assert iv == QUARTERS
    # three fast windows are floored at 0.02: the remainder comes off the free
    # one (0.94 -> 481.28 -> 481), and the missing bin goes to the largest
    iv, _ = WLD.window_optimise(0, QUARTERS, [1.0, 1e6, 1e6, 1e6], [0.25] * 4, 512)
    assert iv == [[1, 482], [483, 492], [493, 502], [503, 512]]
    # ABS(first - last + 1) = 32, 31, 31 bins: 34.04, 32.98, 32.98 -> 34, 33, 33
    iv, _ = WLD.window_optimise(0, [[1, 34], [35, 67], [68, 100]], [5.0] * 3, [1 / 3] * 3, 100)
    assert iv == [[1, 34], [35, 67], [68, 100]]
    # performance outside 0-3, or one window: unchanged
    for args in ((QUARTERS, 4), ([[1, 512]], 0)):
        iv, prev = WLD.window_optimise(0, args[0], [1.0] * len(args[0]), [1.0] * len(args[0]), 512, args[1])
        assert iv == args[0]


def test_window_optimise_settles_rounding_by_descending_size():
    # 100 bins over 3 equal windows of work: 33 each, the extra bin to the first
    iv, _ = WLD.window_optimise(1, [[1, 34], [35, 68], [69, 100]], [1.0, 1.0, 1.0], [1 / 3] * 3, 100)
    sizes = [e - s + 1 for s, e in iv]
    assert sum(sizes) == 100 and iv[0][0] == 1 and iv[-1][1] == 100


def test_sort_descending_is_the_reference_exchange_sort():
    # ties keep the order the exchanges leave (3 before 1), not a stable sort's
    assert WLD.sort_descending([3, 1, 4, 1, 5]) == [4, 2, 0, 3, 1]
    assert WLD.sort_descending([33, 33, 33]) == [0, 1, 2]


def test_nint_and_powi():
    assert [WLD._nint(x) for x in (2.5, -2.5, 0.49999999999999994, 3.4999, 481.28)] == [3, -3, 0, 3, 481]
    for k in range(0, 12):
        y = 1.0
        for _ in range(k):
            y = y * 0.8
        assert abs(WLD._powi(0.8, k) - y) <= 4e-16
    assert WLD._powi(0.8, 3) == (0.8 * 0.8) * 0.8


class FakeStore:
    """The walker-store calls of the drivers, recorded."""

    def __init__(self, open_, windows):
        self.open = open_.copy()
        self.n, self.bins = open_.shape
        self.merged = None
        self.loads = []

    def store_flags(self):
        return self.open.copy()

    def store_merge(self, pick):
        self.merged = np.array(pick)
        for b, p in enumerate(pick):
            self.open[:, b] = p < 0

    def store_load(self, k, b):
        assert not self.open[k, b - 1]
        self.loads.append((k, b))


def test_merge_and_load_draw_like_the_reference():
    """merge_configs draws one holder per bin as ranks_with_config(1 +
    int(u * size)); load_window_config draws min_bin + int(u * (max - min +
    1)) over the walker's window; the draws come in bin then walker order."""
    rng = np.random.default_rng(9)
    open_ = rng.random((4, 20)) < 0.5
    open_[:, 7] = True                     # nobody holds bin 8
    W = FakeStore(open_, None)
    pick = WLD.merge_configs(W, np.random.default_rng(123))
    u = np.random.default_rng(123)
    for b in range(20):
        holders = np.nonzero(~open_[:, b])[0]
        if holders.size:
            assert pick[b] == holders[int(u.random() * holders.size)]
        else:
            assert pick[b] == -1
    assert W.open[:, 7].all()
    assert all(W.open[:, b].all() == (pick[b] < 0) for b in range(20))
    W.open[:] = False                      # after a merge every visited bin is held
    windows = [[1, 12], [9, 20]]
    bins = WLD.load_window_config(W, windows, 2, np.random.default_rng(77))
    u = np.random.default_rng(77)
    for k in range(4):
        s, e = windows[k // 2]
        assert bins[k] == s + int(u.random() * (e - s + 1)) and s <= bins[k] <= e
    assert W.loads == [(k, int(bins[k])) for k in range(4)]


def test_window_optimise_properties_on_random_inputs():
    """Whatever the steps and previous fractions: the windows tile 1..bins
    without gaps, each keeps at least max(INT(0.02 bins), 2) bins, the new
    fractions sum to 1, and create_overlap of the result gives every window
    but the first an overlap with the one below."""
    rng = np.random.default_rng(17)
    for case in range(300):
        nwin = int(rng.integers(2, 9))
        bins = int(rng.integers(8 * nwin, 2000))
        iv = WLD.divide_range(bins, nwin)
        steps = rng.uniform(1e3, 1e7, nwin) * (rng.random(nwin) < 0.9) + 1.0
        prev = rng.dirichlet(np.ones(nwin))
        it = int(rng.integers(0, 6))
        new, frac = WLD.window_optimise(it, iv, steps, prev, bins)
        assert new[0][0] == 1 and new[-1][1] == bins, case
        assert all(new[i][0] == new[i - 1][1] + 1 for i in range(1, nwin)), case
        sizes = [e - s + 1 for s, e in new]
        assert min(sizes) >= max(int(0.02 * bins), 2) and sum(sizes) == bins, case
        assert abs(float(frac.sum()) - 1.0) < 1e-12, case
        idx = WLD.create_overlap(new, 0.25)
        assert all(idx[i][0] <= idx[i - 1][1] for i in range(1, nwin)), case


class FakeWalkers:
    """WangLandauWalkers' interface with scripted answers: every third
    sweeps() call makes every walker flat, histograms are full, and the
    calls are recorded."""

    def __init__(self, walkers, edges):
        self.walkers = [dict(w) for w in walkers]
        self.n, self.bins = len(walkers), len(edges) - 1
        self.log, self.calls, self.enabled = [], 0, False

    def store_enable(self):
        self.enabled = True
        self.log.append("store_enable")

    def enter_windows(self, *a, **k):
        self.log.append("enter_windows")
        return np.arange(self.n, dtype=np.int64) + 10

    def set_config(self, k, cfg):
        pass

    def config(self, k):
        return np.zeros((2, 2, 2), dtype=np.int8)

    def sweeps(self, trials, f, period):
        self.calls += 1
        self.log.append("sweeps")
        return np.zeros(self.n, dtype=np.int64)

    def replica_exchange(self):
        return 0, None, None

    def flatness(self):
        return np.full(self.n, 1.0 if self.calls % 3 == 0 else 0.5)

    def hist(self, k):
        w = self.walkers[k]
        return np.full(w["end_idx"] - w["start_idx"] + 1, 5000.0)

    def set_hist(self, k, h):
        pass

    def reset_hist(self):
        self.log.append("reset_hist")

    def average(self):
        pass

    def dos_combine(self):
        self.log.append("dos_combine")
        return np.zeros(self.bins)

    def set_windows(self, s, e):
        self.log.append(("set_windows", tuple(s), tuple(e)))
        first = {}
        for w in self.walkers:
            first.setdefault(w["window"], len(first))
        for w in self.walkers:
            j = first[w["window"]]
            w["start_idx"], w["end_idx"] = int(s[j]), int(e[j])

    def store_flags(self):
        return np.zeros((self.n, self.bins), dtype=bool)

    def store_merge(self, pick):
        self.log.append("merge")

    def store_load(self, k, b):
        w = self.walkers[k]
        assert w["start_idx"] <= b <= w["end_idx"]
        self.log.append(("load", k))

    def close(self):
        pass


class FakeBatch:
    def __init__(self, chains):
        pass

    def config(self, k):
        return np.zeros((2, 2, 2), dtype=np.int8)

    def close(self):
        pass


def _run_driver(monkeypatch, **kw):
    made = []

    def make(walkers, edges):
        made.append(FakeWalkers(walkers, edges))
        return made[-1]

    monkeypatch.setattr(WLD, "WangLandauWalkers", make)
    monkeypatch.setattr(WLD, "Batch", FakeBatch)
    wl = I.WLParams(mc_sweeps=1, bins=200, num_windows=4, bin_overlap=0.25, tolerance=0.01,
                    flatness=0.8, wl_f=0.05, energy_min=-50.0, energy_max=0.0)
    for k, v in kw.pop("wl", {}).items():
        setattr(wl, k, v)
    setup = B.Setup("bcc", 2, 2, 2, 2, 1)
    out = WLD.wang_landau(setup, np.zeros((2, 2, 1)), np.array([0.0, 0.5, 0.5]), wl, walkers_per_window=2,
                          burn_in="reference", **kw)
    return made[0], out


def test_wang_landau_driver_sequence_with_store_and_windows(monkeypatch):
    """pre-sampling -> mpi_window_optimise(0) -> merge_configs ->
    load_window_config -> histograms reset; then at every ln f step new
    windows and a reload of every walker (performance 0)."""
    W, out = _run_driver(monkeypatch, pre_sample=True)
    log = [x if isinstance(x, str) else x[0] for x in W.log]
    assert log[0] == "store_enable" and W.enabled
    first_sweep = log.index("sweeps")
    assert log.index("store_enable") < first_sweep
    # the end of pre-sampling
    i = log.index("set_windows")
    assert log[i + 1] == "merge" and log[i + 2:i + 2 + W.n] == ["load"] * W.n and log[i + 2 + W.n] == "reset_hist"
    halvings = len(out["record"])
    assert halvings == 3                       # 0.05 -> 0.00625 below 0.01
    assert log.count("set_windows") == 1 + halvings
    assert log.count("load") == W.n * (1 + halvings) and log.count("merge") == 1
    assert len(out["window_sets"]) == 2 + halvings
    for ws in out["window_sets"]:
        assert ws[0][0] == 1 and ws[-1][1] == 200


def test_wang_landau_driver_performance_gates_the_optimiser(monkeypatch):
    # performance 2: the pre-sampling optimisation only (mpi_window_optimise
    # runs for 0-3; the main loop calls it for 0-1)
    W, out = _run_driver(monkeypatch, pre_sample=True, wl={"performance": 2})
    assert [x[0] for x in W.log if not isinstance(x, str)].count("set_windows") == 1
    assert len(out["window_sets"]) == 2
    # no optimisation asked: the windows stay, the reloads still happen
    W, out = _run_driver(monkeypatch, pre_sample=True, optimise_windows=False)
    assert not any(not isinstance(x, str) and x[0] == "set_windows" for x in W.log)
    assert len(out["window_sets"]) == 1 and sum(1 for x in W.log if x[0] == "load") > 0
    # no pre-sampling: no store, no reloads
    W, out = _run_driver(monkeypatch, pre_sample=False)
    assert not W.enabled and not any(x[0] == "load" for x in W.log if not isinstance(x, str))


def test_sweep_blocks_end_at_host_side_samples():
    """The annealing drivers run the sweeps between host-side samples as one
    device block: a block ends at the first sweep after which ASRO or ALRO
    is sampled, else at the temperature's last sweep."""
    m = I.MetropolisParams(mode="simulated_annealing", n_mc_steps=10 * 8, n_sample_steps=8,
                           calculate_energies=True, calculate_asro=True, n_sample_steps_asro=3 * 8,
                           n_sample_steps_trajectory=8, T=300.0, T_steps=1, delta_T=0.0)

    def blocks(m, n_sweeps=10, step=8):
        out, i = [], 1
        while i <= n_sweeps:
            e = M._block_end(m, i, n_sweeps, step)
            out.append((i, e))
            i = e + 1
        return out

    assert blocks(m) == [(1, 3), (4, 6), (7, 9), (10, 10)]
    m.calculate_asro = False
    assert blocks(m) == [(1, 10)]
    m.calculate_alro = True
    m.n_sample_steps_alro = 4 * 8
    assert blocks(m) == [(1, 4), (5, 8), (9, 10)]
    m.calculate_asro = True
    assert blocks(m) == [(1, 3), (4, 4), (5, 6), (7, 8), (9, 9), (10, 10)]
