"""GPU Wang-Landau walker updates against the oracle: sweeps() of every
walker followed by the in-window average (walker order), bit for bit --
ln g, histograms, configurations, accepted moves and the streams."""
import numpy as np
import pytest

import brawl_gb300 as B
from oracle import oracle as O
from tests.test_gpu_metropolis import conc_vector, random_V

pytestmark = pytest.mark.gpu


def _emulate(mods, cfgs, rngs, walkers, bin_edges, lngs, hists, n_trials, wl_f, period):
    bins = bin_edges.size - 1
    acc = []
    for k, w in enumerate(walkers):
        e = mods[k].total_energy(cfgs[k])
        a, _, _ = mods[k].wl_sweep(cfgs[k], rngs[k], bin_edges, lngs[k], hists[k], e, bins,
                                   w["start_idx"], w["end_idx"], n_trials, wl_f, period,
                                   nbr_swap=w.get("nbr_swap", False))
        acc.append(a)
    windows = sorted(set(w["window"] for w in walkers))
    for win in windows:
        idx = [k for k, w in enumerate(walkers) if w["window"] == win]
        if len(idx) < 2:
            continue
        inv = float(np.float32(len(idx)))
        for arrs in (lngs, hists):
            s = arrs[idx[0]].copy()
            for k in idx[1:]:
                s = s + arrs[k]
            s = s / inv
            for k in idx:
                arrs[k][:] = s
    return acc


@pytest.mark.parametrize("lattice,n,ns,nsh,windows,nbr", [
    ("bcc", (4, 4, 4), 4, 6, [(1, 30), (19, 48)], False),
    ("fcc", (3, 3, 3), 3, 3, [(10, 30), (20, 40), (18, 44)], False),
    ("bcc", (4, 4, 4), 4, 6, [(1, 30), (19, 48)], True),
    ("fcc", (3, 3, 3), 3, 3, [(10, 30), (20, 40), (18, 44)], True),
])
def test_wang_landau_sweeps_match_oracle(lattice, n, ns, nsh, windows, nbr):
    rng = np.random.default_rng(21)
    V = random_V(rng, ns, nsh)
    setup = B.Setup(lattice, *n, ns, nsh)
    mod0 = O.OracleModel(lattice, *n, V)
    walkers, mods, cfgs, rngs = [], [], [], []
    r0 = O.OracleRng(4242)
    for win, (lo, hi) in enumerate(windows):
        for rep in range(2):
            cfg, _ = mod0.initial_setup(r0, conc_vector(ns))
            seed = 110179 + 11 * len(walkers)
            walkers.append(dict(setup=setup, V=V, seed=seed, config=cfg.copy(), start_idx=lo,
                                end_idx=hi, window=win, nbr_swap=nbr))
            mods.append(O.OracleModel(lattice, *n, V))
            cfgs.append(cfg.copy())
            rngs.append(O.OracleRng(seed))
    E = np.array([mod0.total_energy(c) for c in cfgs])
    bins = 48
    # bins around the walkers' energies so each starts inside every window
    half = max(float(np.ptp(E)), 0.02) * 4.0
    mid = float(E.mean())
    bin_edges = mid - half + (np.arange(bins + 1) * (2 * half / bins))
    bidx = [O.wl_bin_index(e, bin_edges, bins) for e in E]
    assert all(lo <= b <= hi for b, (lo, hi) in zip(bidx, [windows[w["window"]] for w in walkers]))
    lngs = [np.zeros(bins) for _ in walkers]
    hists = [np.zeros(w["end_idx"] - w["start_idx"] + 1) for w in walkers]
    wl = B.WangLandauWalkers(walkers, bin_edges)
    wl_f = float(np.float32(0.05))
    period = int(0.02 * float(np.float32(setup.n_atoms)))
    for call in range(3):
        acc_o = _emulate(mods, cfgs, rngs, walkers, bin_edges, lngs, hists, 700, wl_f, period)
        acc_g = wl.sweeps(700, wl_f, period)
        assert list(acc_g) == acc_o
        for k in range(len(walkers)):
            assert np.array_equal(wl.lng(k), lngs[k])
            assert np.array_equal(wl.hist(k), hists[k])
            assert np.array_equal(wl.config(k), cfgs[k])
    for k in range(len(walkers)):
        assert np.array_equal(wl.genrand(k, 20), np.array([rngs[k].uniform() for _ in range(20)]))
    assert np.array_equal(wl.energies(), np.array([mods[k].total_energy(cfgs[k]) for k in range(len(walkers))]))


def test_wang_landau_walker_outside_window_is_reported():
    rng = np.random.default_rng(3)
    V = random_V(rng, 2, 2)
    setup = B.Setup("bcc", 3, 3, 3, 2, 2)
    mod = O.OracleModel("bcc", 3, 3, 3, V)
    cfg, _ = mod.initial_setup(O.OracleRng(5), conc_vector(2))
    e = mod.total_energy(cfg)
    bin_edges = e + 1.0 + np.arange(11) * 0.1      # every bin above the walker
    wl = B.WangLandauWalkers([dict(setup=setup, V=V, seed=1, config=cfg, start_idx=1,
                                   end_idx=10, window=0)], bin_edges)
    with pytest.raises(B.BrawlError) as ex:
        wl.sweeps(10, 0.05, 1)
    assert ex.value.code == 6


def _exchange_system(lattice, n, ns, nsh, n_windows, per_window, bins, seed):
    """Walkers spread over n_windows overlapping windows of `bins` bins, each
    starting inside its window; bin edges spanning a pool of random
    configurations' energies."""
    rng = np.random.default_rng(seed)
    V = random_V(rng, ns, nsh)
    setup = B.Setup(lattice, *n, ns, nsh)
    mod0 = O.OracleModel(lattice, *n, V)
    r0 = O.OracleRng(seed + 1)
    pool = [mod0.initial_setup(r0, conc_vector(ns))[0] for _ in range(160)]
    E = np.array([mod0.total_energy(c) for c in pool])
    lo_e, hi_e = float(E.min()), float(E.max())
    pad = 1e-3 * (hi_e - lo_e)
    bin_edges = (lo_e - pad) + np.arange(bins + 1) * ((hi_e - lo_e + 2 * pad) / bins)
    # windows of equal width, each overlapping the next by half its width
    width = (2 * bins) // (n_windows + 1)
    starts = [1 + k * (width // 2) for k in range(n_windows)]
    ends = [s + width - 1 for s in starts]
    ends[-1] = bins
    bidx = np.array([O.wl_bin_index(e, bin_edges, bins) for e in E])
    used, walkers = set(), []
    for k in range(n_windows):
        # prefer configurations in the overlaps so exchanges are attempted
        cand = [i for i in range(len(pool)) if starts[k] <= bidx[i] <= ends[k] and i not in used]
        cand.sort(key=lambda i: min(bidx[i] - starts[k], ends[k] - bidx[i]))
        assert len(cand) >= per_window
        for i in cand[:per_window]:
            used.add(i)
            walkers.append(dict(setup=setup, V=V, seed=110179 + 11 * len(walkers),
                                config=pool[i].copy(), start_idx=starts[k], end_idx=ends[k],
                                window=k))
    return setup, V, walkers, bin_edges, starts, ends


@pytest.mark.parametrize("lattice,n,ns,nsh,n_windows,per_window", [
    ("bcc", (4, 4, 4), 4, 4, 4, 3),
    ("fcc", (3, 3, 3), 3, 3, 3, 4),
])
def test_wang_landau_exchange_flatness_combine_match_oracle(lattice, n, ns, nsh, n_windows, per_window):
    bins = 60
    setup, V, walkers, bin_edges, starts, ends = _exchange_system(lattice, n, ns, nsh, n_windows,
                                                                  per_window, bins, 77)
    mods = [O.OracleModel(lattice, *n, V) for _ in walkers]
    cfgs = [w["config"].copy() for w in walkers]
    rngs = [O.OracleRng(w["seed"]) for w in walkers]
    lngs = [np.zeros(bins) for _ in walkers]
    hists = [np.zeros(w["end_idx"] - w["start_idx"] + 1) for w in walkers]
    wl = B.WangLandauWalkers(walkers, bin_edges)
    wl_f = 1.0
    period = max(1, int(0.02 * float(np.float32(setup.n_atoms))))
    total_acc = 0
    for it in range(6):
        acc_o = _emulate(mods, cfgs, rngs, walkers, bin_edges, lngs, hists, 400, wl_f, period)
        assert list(wl.sweeps(400, wl_f, period)) == acc_o
        E = [mods[k].total_energy(cfgs[k]) for k in range(len(walkers))]
        na_o, partner_o, exch_o = O.wl_replica_exchange(starts, ends, per_window, bin_edges, E, lngs,
                                                        rngs, cfgs)
        na_g, partner_g, exch_g = wl.replica_exchange()
        assert na_g == na_o
        assert np.array_equal(partner_g, partner_o)
        assert np.array_equal(exch_g, exch_o)
        for k in range(len(walkers)):
            assert np.array_equal(wl.config(k), cfgs[k])
        total_acc += na_o
        flat_o = np.array([O.wl_flatness(h) for h in hists])
        assert np.array_equal(wl.flatness(), flat_o)
    assert (partner_o >= 0).any()
    for k in range(len(walkers)):
        assert np.array_equal(wl.genrand(k, 8), np.array([rngs[k].uniform() for _ in range(8)]))
    # dos_average then dos_combine, as at the end of a Wang-Landau iteration
    wl.average()
    for k0 in range(0, len(walkers), per_window):
        idx = list(range(k0, k0 + per_window))
        s = lngs[idx[0]].copy()
        for k in idx[1:]:
            s = s + lngs[k]
        s = s / float(np.float32(per_window))
        for k in idx:
            lngs[k][:] = s
    for k in range(len(walkers)):
        assert np.array_equal(wl.lng(k), lngs[k])
    comb_o = O.wl_dos_combine(starts, ends, np.stack([lngs[k] for k in range(0, len(walkers), per_window)]))
    comb_g = wl.dos_combine()
    assert np.array_equal(comb_g, comb_o)
    for k in range(len(walkers)):
        assert np.array_equal(wl.lng(k), comb_o)
    wl.reset_hist()
    assert not wl.hist(0).any()


def test_wang_landau_exchange_needs_equal_windows():
    rng = np.random.default_rng(5)
    V = random_V(rng, 2, 2)
    setup = B.Setup("bcc", 3, 3, 3, 2, 2)
    mod = O.OracleModel("bcc", 3, 3, 3, V)
    r = O.OracleRng(9)
    cfgs = [mod.initial_setup(r, conc_vector(2))[0] for _ in range(3)]
    e = [mod.total_energy(c) for c in cfgs]
    bin_edges = min(e) - 1.0 + np.arange(21) * ((max(e) - min(e) + 2.0) / 20)
    ws = [dict(setup=setup, V=V, seed=k + 1, config=cfgs[k], start_idx=1, end_idx=20,
               window=0 if k < 2 else 1) for k in range(3)]
    wl = B.WangLandauWalkers(ws, bin_edges)
    with pytest.raises(B.BrawlError) as ex:
        wl.replica_exchange()
    assert ex.value.code == 1


@pytest.mark.parametrize("nbr", [False, True])
def test_wang_landau_radial_samples_match_oracle(nbr):
    """sweeps() with the radial-density samples (src/wang-landau.F90:566-586):
    radial_record, rho_of_E and radial_mc_steps per walker equal the
    oracle's, bit for bit, also after radial_record_bool marks some bins and
    once every bin is marked (rho_saved)."""
    rng = np.random.default_rng(33)
    lattice, n, ns, nsh, wc = "bcc", (4, 4, 4), 4, 6, 3
    V = random_V(rng, ns, nsh)
    setup = B.Setup(lattice, *n, ns, nsh)
    mod0 = O.OracleModel(lattice, *n, V)
    windows = [(1, 30), (19, 48)]
    walkers, mods, cfgs, rngs = [], [], [], []
    r0 = O.OracleRng(777)
    for win, (lo, hi) in enumerate(windows):
        for rep in range(2):
            cfg, _ = mod0.initial_setup(r0, conc_vector(ns))
            seed = 110179 + 11 * len(walkers)
            walkers.append(dict(setup=setup, V=V, seed=seed, config=cfg.copy(), start_idx=lo,
                                end_idx=hi, window=win, nbr_swap=nbr))
            mods.append(O.OracleModel(lattice, *n, V))
            cfgs.append(cfg.copy())
            rngs.append(O.OracleRng(seed))
    E = np.array([mod0.total_energy(c) for c in cfgs])
    bins = 48
    half = max(float(np.ptp(E)), 0.02) * 4.0
    bin_edges = float(E.mean()) - half + (np.arange(bins + 1) * (2 * half / bins))
    shells = mod0.lattice_shells(cfgs[0], wc)
    radial_samples, num_walkers = 5, 2
    cap = max(radial_samples // num_walkers, 1)
    done = np.zeros(bins, dtype=np.uint8)
    rads = [{"shells": np.ascontiguousarray(shells), "cap": cap, "done": done,
             "record": np.zeros(bins, dtype=np.int32), "rho_of_E": np.zeros((bins, wc, ns, ns)),
             "steps": np.zeros(1, dtype=np.int32)} for _ in walkers]
    lngs = [np.zeros(bins) for _ in walkers]
    hists = [np.zeros(w["end_idx"] - w["start_idx"] + 1) for w in walkers]
    wl = B.WangLandauWalkers(walkers, bin_edges)
    wl.radial_enable(wc, shells, radial_samples, num_walkers)
    wl_f = float(np.float32(0.05))
    period = int(0.02 * float(np.float32(setup.n_atoms)))
    for call in range(4):
        if call == 2:
            done[::3] = 1                    # save_rho_E marked some bins
            wl.radial_set_done(done)
        if call == 3:
            done[:] = 1                      # rho_saved: no more samples
            wl.radial_set_done(done)
        acc_o = []
        for k, w in enumerate(walkers):
            e = mods[k].total_energy(cfgs[k])
            a, _, _ = mods[k].wl_sweep(cfgs[k], rngs[k], bin_edges, lngs[k], hists[k], e, bins,
                                       w["start_idx"], w["end_idx"], 1500, wl_f, period, nbr_swap=nbr,
                                       radial=None if call == 3 else rads[k])
            acc_o.append(a)
        for win in range(len(windows)):
            idx = [k for k, w in enumerate(walkers) if w["window"] == win]
            inv = float(np.float32(len(idx)))
            for arrs in (lngs, hists):
                s = arrs[idx[0]].copy()
                for k in idx[1:]:
                    s = s + arrs[k]
                s = s / inv
                for k in idx:
                    arrs[k][:] = s
        acc_g = wl.sweeps(1500, wl_f, period)
        assert list(acc_g) == acc_o
        for k in range(len(walkers)):
            rec, rho, steps = wl.radial(k)
            assert np.array_equal(rec, rads[k]["record"]), (call, k)
            assert np.array_equal(rho, rads[k]["rho_of_E"]), (call, k)
            assert steps == int(rads[k]["steps"][0]), (call, k)
            assert np.array_equal(wl.config(k), cfgs[k])
            assert np.array_equal(wl.lng(k), lngs[k])
    assert sum(int(r["record"].sum()) for r in rads) > 8


def test_enter_windows_match_oracle():
    """enter_energy_window on the device (brawl_wl_enter_windows, starting
    from initial_setup on each walker's stream) against the oracle's walk:
    iterations, configuration, energy and stream of every walker."""
    rng = np.random.default_rng(44)
    lattice, n, ns, nsh = "bcc", (4, 4, 4), 3, 4
    V = random_V(rng, ns, nsh)
    setup = B.Setup(lattice, *n, ns, nsh)
    mod = O.OracleModel(lattice, *n, V)
    conc = conc_vector(ns)
    nums = None
    c0, _ = mod.initial_setup(O.OracleRng(1), conc, nums)
    E = np.array([mod.total_energy(mod.initial_setup(O.OracleRng(s), conc, nums)[0]) for s in range(20)])
    bins = 40
    half = max(float(np.ptp(E)), 0.02) * 1.5
    edges = float(E.mean()) - half + np.arange(bins + 1) * (2 * half / bins)
    windows = [(1, 22), (19, 40)]
    walkers = []
    for win, (lo, hi) in enumerate(windows):
        for rep in range(2):
            walkers.append(dict(setup=setup, V=V, seed=110179 + 11 * len(walkers), config=c0, start_idx=lo,
                                end_idx=hi, window=win))
    e_min_mev, e_max_mev = -30.0, 20.0
    W = B.WangLandauWalkers(walkers, edges)
    steps = W.enter_windows(e_min_mev, e_max_mev, conc, nums, initial=True, max_steps=2_000_000)
    f32 = np.float32
    x4 = (f32(0.0025) * abs(f32(e_max_mev) - f32(e_min_mev))) * f32(setup.n_atoms)
    x = float(x4) / (13.605693122 * 1000.0)
    sig2x2 = 2.0 * (x * x)
    for k, w in enumerate(walkers):
        r = O.OracleRng(w["seed"])
        cfg, _ = mod.initial_setup(r, conc, nums)
        it, e = mod.wl_enter_window(cfg, r, conc, nums, edges[w["start_idx"] - 1], edges[w["end_idx"]],
                                    sig2x2, 2_000_000)
        assert it > 0 and steps[k] == it, k
        assert np.array_equal(W.config(k), cfg), k
        assert W.energies()[k] == e
        assert np.array_equal(W.genrand(k, 10), np.array([r.uniform() for _ in range(10)])), k


def test_wang_landau_store_merge_windows_match_oracle():
    """The configuration store of sweeps() (config_per_bin / config_store),
    merge_configs' copies, load_window_config and new windows against the
    oracle: flags, every stored configuration, ln g, histograms,
    configurations and accepted moves, bit for bit, before and after the
    windows change."""
    lattice, n, ns, nsh = "bcc", (4, 4, 4), 4, 6
    windows = [(1, 30), (19, 48)]
    rng = np.random.default_rng(33)
    V = random_V(rng, ns, nsh)
    setup = B.Setup(lattice, *n, ns, nsh)
    mod0 = O.OracleModel(lattice, *n, V)
    walkers, mods, cfgs, rngs = [], [], [], []
    r0 = O.OracleRng(977)
    for win, (lo, hi) in enumerate(windows):
        for rep in range(2):
            cfg, _ = mod0.initial_setup(r0, conc_vector(ns))
            seed = 110179 + 11 * len(walkers)
            walkers.append(dict(setup=setup, V=V, seed=seed, config=cfg.copy(), start_idx=lo,
                                end_idx=hi, window=win))
            mods.append(O.OracleModel(lattice, *n, V))
            cfgs.append(cfg.copy())
            rngs.append(O.OracleRng(seed))
    E = np.array([mod0.total_energy(c) for c in cfgs])
    bins = 48
    half = max(float(np.ptp(E)), 0.02) * 4.0
    bin_edges = float(E.mean()) - half + (np.arange(bins + 1) * (2 * half / bins))
    nw = len(walkers)
    lngs = [np.zeros(bins) for _ in walkers]
    hists = [np.zeros(w["end_idx"] - w["start_idx"] + 1) for w in walkers]
    stores = [dict(slots=np.zeros((bins,) + cfgs[0].shape, dtype=np.int8), open=np.ones(bins, dtype=np.uint8))
              for _ in walkers]
    wl = B.WangLandauWalkers(walkers, bin_edges)
    wl.store_enable()
    wl_f = float(np.float32(0.05))
    period = int(0.02 * float(np.float32(setup.n_atoms)))

    def run_calls(calls):
        for _ in range(calls):
            acc_o = []
            for k, w in enumerate(walkers):
                e = mods[k].total_energy(cfgs[k])
                a, _, _ = mods[k].wl_sweep(cfgs[k], rngs[k], bin_edges, lngs[k], hists[k], e, bins,
                                           w["start_idx"], w["end_idx"], 600, wl_f, period, store=stores[k])
                acc_o.append(a)
            for win in range(len(windows)):
                idx = [k for k, w in enumerate(walkers) if w["window"] == win]
                for arrs in (lngs, hists):
                    s = arrs[idx[0]].copy()
                    for k in idx[1:]:
                        s = s + arrs[k]
                    s = s / float(np.float32(len(idx)))
                    for k in idx:
                        arrs[k][:] = s
            assert list(wl.sweeps(600, wl_f, period)) == acc_o
        check_all()

    def check_all():
        flags = wl.store_flags()
        for k in range(nw):
            assert np.array_equal(flags[k], stores[k]["open"].astype(bool)), k
            for b in np.nonzero(~flags[k])[0]:
                assert np.array_equal(wl.store_config(k, int(b) + 1), stores[k]["slots"][b]), (k, b)
            assert np.array_equal(wl.lng(k), lngs[k])
            assert np.array_equal(wl.hist(k), hists[k])
            assert np.array_equal(wl.config(k), cfgs[k])

    run_calls(2)
    closed = [np.nonzero(stores[k]["open"] == 0)[0] for k in range(nw)]
    assert all(c.size > 0 for c in closed)
    # an open bin holds nothing to load; a non-holder cannot be picked
    open_bin = int(np.nonzero(stores[0]["open"])[0][0]) + 1 if stores[0]["open"].any() else None
    if open_bin is not None:
        with pytest.raises(B.BrawlError, match="holds no stored configuration"):
            wl.store_load(0, open_bin)
        bad = np.full(bins, -1, dtype=np.int32)
        bad[open_bin - 1] = 0
        with pytest.raises(B.BrawlError, match="holds no configuration"):
            wl.store_merge(bad)

    # merge_configs with a drawn holder per bin
    pick = np.full(bins, -1, dtype=np.int32)
    draw = np.random.default_rng(5)
    for b in range(bins):
        holders = [k for k in range(nw) if stores[k]["open"][b] == 0]
        if holders:
            pick[b] = holders[int(draw.random() * len(holders))]
    wl.store_merge(pick)
    for b in range(bins):
        src = pick[b] if pick[b] >= 0 else 0
        for k in range(nw):
            if k != src:
                stores[k]["slots"][b] = stores[src]["slots"][b]
            stores[k]["open"][b] = 0 if pick[b] >= 0 else 1
    check_all()

    # new windows (the histograms restart), then a stored configuration of
    # each walker's new window
    new = [(1, 26), (20, 48)]
    with pytest.raises(B.BrawlError, match="outside 1..bins"):
        wl.set_windows([1, 20], [26, 49])
    wl.set_windows([s for s, _ in new], [e for _, e in new])
    for k, w in enumerate(walkers):
        w["start_idx"], w["end_idx"] = new[w["window"]]
        hists[k] = np.zeros(w["end_idx"] - w["start_idx"] + 1)
    for k, w in enumerate(walkers):
        inside = [b for b in range(w["start_idx"], w["end_idx"] + 1) if stores[k]["open"][b - 1] == 0]
        assert inside
        b = inside[int(draw.random() * len(inside))]
        wl.store_load(k, b)
        cfgs[k] = stores[k]["slots"][b - 1].copy()
        assert O.wl_bin_index(mod0.total_energy(cfgs[k]), bin_edges, bins) == b
    check_all()
    run_calls(2)


def test_wang_landau_divided_windows_exchange_match_oracle():
    """The Wang-Landau workload's layout, reduced: bcc 6^3, 4 species, 4
    shells, the bins of create_energy_bins split by divide_range into 8
    windows extended by create_overlap (bin overlap 0.25), 4 walkers per
    window placed in their windows by the driver's temperature search; then
    cycles of sweeps() and replica exchange between adjacent windows, the
    device against the oracle bit for bit (ln g, histograms, partners,
    exchanges, configurations, streams)."""
    from brawl_gb300 import wang_landau as WLD
    lattice, n, ns, nsh, nwin, per_window, bins = "bcc", (6, 6, 6), 4, 4, 8, 4, 400
    rng = np.random.default_rng(91)
    V = random_V(rng, ns, nsh)
    setup = B.Setup(lattice, *n, ns, nsh)
    N = setup.n_atoms
    conc = conc_vector(ns)
    pilot = B.Batch([dict(setup=setup, V=V, seed=5 + k, beta=1.0 / (T * B.K_B_IN_RY),
                          species_concentrations=conc) for k, T in enumerate([300.0, 1e12])])
    pilot.metropolis(200 * N)
    E = pilot.total_energy()
    pilot.close()
    to_mev = B.RY_TO_EV * 1000.0 / N
    emin, emax = float(np.float32(E[0] * to_mev)), float(np.float32(E[1] * to_mev))
    edges = WLD.create_energy_bins(N, emin, emax, bins)
    windows = WLD.create_overlap(WLD.divide_range(bins, nwin), float(np.float32(0.25)))
    starts, ends = [w[0] for w in windows], [w[1] for w in windows]
    nw = nwin * per_window
    seeds = [110179 + 11 * r for r in range(nw)]
    targets = []
    for r in range(nw):
        s, e = windows[r // per_window]
        lo_e, hi_e = edges[s - 1], edges[e]
        c = abs(hi_e - lo_e) * 0.1
        targets.append((lo_e + c, hi_e - c))
    cfgs0, _ = WLD._burn_in(setup, V, [1000 + r for r in range(nw)], conc, targets, N)
    walkers = [dict(setup=setup, V=V, seed=seeds[r], config=cfgs0[r], start_idx=starts[r // per_window],
                    end_idx=ends[r // per_window], window=r // per_window) for r in range(nw)]
    mods = [O.OracleModel(lattice, *n, V) for _ in walkers]
    cfgs = [w["config"].copy() for w in walkers]
    rngs = [O.OracleRng(w["seed"]) for w in walkers]
    lngs = [np.zeros(bins) for _ in walkers]
    hists = [np.zeros(w["end_idx"] - w["start_idx"] + 1) for w in walkers]
    wl = B.WangLandauWalkers(walkers, edges)
    period = int(0.02 * float(np.float32(N)))
    attempted = 0
    for cycle in range(4):
        acc_o = _emulate(mods, cfgs, rngs, walkers, edges, lngs, hists, 1000, 1.0, period)
        assert list(wl.sweeps(1000, 1.0, period)) == acc_o
        Es = [mods[k].total_energy(cfgs[k]) for k in range(nw)]
        na_o, partner_o, exch_o = O.wl_replica_exchange(starts, ends, per_window, edges, Es, lngs,
                                                        rngs, cfgs)
        na_g, partner_g, exch_g = wl.replica_exchange()
        assert na_g == na_o
        assert np.array_equal(partner_g, partner_o)
        assert np.array_equal(exch_g, exch_o)
        attempted += int((partner_o >= 0).sum())
        for k in range(nw):
            assert np.array_equal(wl.config(k), cfgs[k])
            assert np.array_equal(wl.lng(k), lngs[k])
            assert np.array_equal(wl.hist(k), hists[k])
    assert attempted > 0
    for k in range(nw):
        assert np.array_equal(wl.genrand(k, 8), np.array([rngs[k].uniform() for _ in range(8)]))
