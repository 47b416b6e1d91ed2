"""The oracle's Wang-Landau exchange, stitching and flatness
(src/wang-landau.F90:222, 1147-1194, 1392-1525) against an independent
pure-Python restatement of the same reference lines, plus hand-worked
cases.  CPU only."""
import math

import numpy as np
import pytest

from oracle import oracle as O


def _py_bin(e, edges, bins):
    return int(((e - edges[0]) / (edges[bins] - edges[0])) * bins) + 1


def _py_exchange(ws, we, pw, edges, E, lngs, rng_words, cfgs):
    """replica_exchange + shuffle_rows written out directly from the
    reference; rng_words[w] is a callable returning walker w's next
    genrand()."""
    nwin = len(ws)
    bins = len(edges) - 1
    n = nwin * pw
    ib, ov = [], []
    for w in range(n):
        idx = w // pw + 1
        b = _py_bin(E[w], edges, bins)
        lower = idx > 1 and b < we[idx - 2] + 1 and b > ws[idx - 1] - 1
        upper = idx < nwin and b > ws[idx] - 1 and b < we[idx - 1] + 1
        ib.append(b)
        ov.append([w, idx if upper else (idx - 1 if lower else 0)])
    partner, acc = [-1] * n, [0] * n
    for i in range(1, nwin):
        lo = [list(r) for r in ov[(i - 1) * pw:i * pw]]
        up = [list(r) for r in ov[i * pw:(i + 1) * pw]]
        for arr in (lo, up):
            for r in range(pw, 1, -1):
                k = min(1 + int(rng_words[0]() * r), pw)
                arr[r - 1], arr[k - 1] = arr[k - 1], arr[r - 1]
        ex = []
        for j in range(pw):
            if lo[j][1] == 0:
                continue
            for k in range(pw):
                if up[k][1] == 0:
                    continue
                if lo[j][1] == up[k][1]:
                    ex.append((lo[j][0], up[k][0]))
                    lo[j] = [0, 0]
                    up[k] = [0, 0]
        for a, b in ex:
            jb = _py_bin(E[b], edges, bins)
            partner[a], partner[b] = b, a
            if rng_words[a]() < math.exp(lngs[a][ib[a] - 1] - lngs[a][jb - 1]):
                cfgs[a], cfgs[b] = cfgs[b].copy(), cfgs[a].copy()
                acc[a] = acc[b] = 1
    return sum(acc) // 2, partner, acc


@pytest.mark.parametrize("nwin,pw,seed", [(2, 2, 1), (4, 3, 2), (5, 4, 3), (3, 6, 4)])
def test_exchange_matches_python_restatement(nwin, pw, seed):
    rng = np.random.default_rng(seed)
    bins = 40
    width = (2 * bins) // (nwin + 1)
    ws = [1 + k * (width // 2) for k in range(nwin)]
    we = [s + width - 1 for s in ws]
    we[-1] = bins
    edges = np.linspace(-1.0, 1.0, bins + 1)
    n = nwin * pw
    E = []
    for w in range(n):
        k = w // pw
        b = int(rng.integers(ws[k], we[k] + 1))
        E.append(float(edges[b - 1] + 0.5 * (edges[b] - edges[b - 1])))
    lngs = [rng.uniform(0, 3, bins) for _ in range(n)]
    cfgs = [rng.integers(1, 4, 16).astype(np.int8) for _ in range(n)]
    r_c = [O.OracleRng(1000 + w) for w in range(n)]
    r_p = [O.OracleRng(1000 + w) for w in range(n)]
    cfg_c = [c.copy() for c in cfgs]
    cfg_p = [c.copy() for c in cfgs]
    na, partner, acc = O.wl_replica_exchange(ws, we, pw, edges, E, lngs, r_c, cfg_c)
    na_p, partner_p, acc_p = _py_exchange(ws, we, pw, edges, E, lngs, [r.uniform for r in r_p], cfg_p)
    assert na == na_p
    assert list(partner) == partner_p
    assert list(acc) == acc_p
    for a, b in zip(cfg_c, cfg_p):
        assert np.array_equal(a, b)
    for a, b in zip(r_c, r_p):
        assert np.array_equal(a.state_words(), b.state_words())


def test_exchange_shuffles_draw_from_walker_zero():
    """Every adjacent pair of windows shuffles two lists of pw rows on rank
    0's stream: 2 (pw - 1) draws each, whether or not anything matches."""
    nwin, pw, bins = 4, 3, 40
    ws, we = [1, 11, 21, 31], [10, 20, 30, 40]     # no overlaps: nothing matches
    edges = np.linspace(0.0, 1.0, bins + 1)
    E = [float(edges[ws[w // pw] + 2]) for w in range(nwin * pw)]
    rngs = [O.OracleRng(7 + w) for w in range(nwin * pw)]
    ref = O.OracleRng(7)
    cfgs = [np.zeros(4, np.int8) for _ in range(nwin * pw)]
    na, partner, acc = O.wl_replica_exchange(ws, we, pw, edges, E, [np.zeros(bins)] * (nwin * pw),
                                             rngs, cfgs)
    assert na == 0 and (partner == -1).all()
    for _ in range(2 * (pw - 1) * (nwin - 1)):
        ref.uniform()
    assert np.array_equal(rngs[0].state_words(), ref.state_words())
    assert np.array_equal(rngs[1].state_words(), O.OracleRng(8).state_words())


def test_dos_combine_hand_case():
    lw = np.array([[0, 1, 2, 3, 4, 5, 6, 0, 0, 0],
                   [0, 0, 0, 10, 11, 12.5, 13, 14, 15, 16]], dtype=np.float64)
    out = O.wl_dos_combine([1, 4], [6, 10], lw)
    # overlap bins 4..6: slopes agree at bin 4->5, so bins 5..10 follow
    # window 2 shifted by 4 - 11
    assert np.array_equal(out, [0, 1, 2, 3, 4, 5.5, 6, 7, 8, 9])


def test_dos_combine_rounds_like_the_reference_loop():
    rng = np.random.default_rng(11)
    bins = 30
    ws, we = [1, 8, 16], [12, 20, 30]
    lw = rng.uniform(-5, 5, (3, bins)).cumsum(axis=1)
    out = O.wl_dos_combine(ws, we, lw)
    comb = lw[0].copy()
    beta_index = 0
    for i in range(2, 4):
        buf = lw[i - 1]
        s, e = ws[i - 1], we[i - 1]
        diff = np.finfo(np.float64).max
        for j in range(0, we[i - 2] - ws[i - 1]):
            bo = comb[s + j] - comb[s + j - 1]
            bm = buf[s + j] - buf[s + j - 1]
            if abs(bo - bm) < diff:
                diff = abs(bo - bm)
                beta_index = s + j + 1
        for j in range(beta_index, e + 1):
            comb[j - 1] = buf[j - 1] + comb[beta_index - 1] - buf[beta_index - 1]
    comb = comb - comb.min()
    assert np.array_equal(out, comb)


def test_dos_combine_without_overlap_is_an_error():
    with pytest.raises(ValueError):
        O.wl_dos_combine([1, 6], [5, 10], np.zeros((2, 10)))


def test_flatness():
    assert O.wl_flatness([2.0, 4.0, 6.0]) == 2.0 / 4.0
    h = np.array([0.25, 0.5, 0.75, 1.0])
    assert O.wl_flatness(h) == 0.25 / (2.5 / 4)


def test_windows_and_bins_follow_the_reference():
    """divide_range / create_overlap / create_energy_bins for the golden
    inputs (512 bins, 4 windows, 25% overlap, -96..0 meV/atom, 128 atoms)."""
    from brawl_gb300 import wang_landau as W
    assert W.divide_range(512, 4) == [[1, 128], [129, 256], [257, 384], [385, 512]]
    assert W.create_overlap(W.divide_range(512, 4), 0.25) == [[1, 128], [97, 256], [217, 384], [343, 512]]
    e = W.create_energy_bins(128, -96.0, 0.0, 512)
    assert e.size == 513 and e[0] == -96.0 * 128 / (13.605693122 * 1000.0) and abs(e[-1]) < 1e-15


BCC_NBRS = [(1, 1, 1), (1, 1, -1), (1, -1, 1), (1, -1, -1), (-1, 1, 1), (-1, 1, -1), (-1, -1, 1),
            (-1, -1, -1)]


def _py_sweeps_nbr(mod, n, cfg, rng, edges, lng, hist, e, bins, start, end, n_trials, f, period,
                   nbr=True, radial=None, store=None):
    """sweeps (src/wang-landau.F90:539-632) with select_sites_nbr (:1527-1532)
    or select_sites, the radial-density samples (:566-586) and the
    configuration store (:605-622), written out from the reference, on a bcc
    lattice n x n x n; the site draw, the pair energies and radial_densities
    come from the oracle."""
    W = 2 * n
    n_atoms = 2 * n ** 3
    acc = 0
    for i in range(1, n_trials + 1):
        a = mod.random_site(rng)
        if nbr:
            k = int(math.floor(8.0 * rng.uniform()))      # bcc_random_nbr: floor(8 u) + 1
            d = BCC_NBRS[k]
            b = tuple((a[c] + d[c]) % W for c in range(3))
        else:
            b = mod.random_site(rng)
        s1, s2 = cfg[a[2], a[1], a[0]], cfg[b[2], b[1], b[0]]
        p_un = mod.pair_energy(cfg, a, b)
        cfg[a[2], a[1], a[0]], cfg[b[2], b[1], b[0]] = s2, s1
        e_sw = e
        if s1 != s2:
            e_sw = e - p_un + mod.pair_energy(cfg, a, b)
        ib, jb = _py_bin(e, edges, bins), _py_bin(e_sw, edges, bins)
        if radial is not None and 0 < jb < bins + 1:
            if radial["record"][jb - 1] < radial["cap"] and not radial["done"][jb - 1]:
                radial["steps"][0] += 1
                if radial["steps"][0] >= n_atoms:
                    radial["steps"][0] = 0
                    radial["record"][jb - 1] += 1
                    rho, _ = mod.radial_densities(cfg, radial["shells"])
                    radial["rho_of_E"][jb - 1] = radial["rho_of_E"][jb - 1] + rho
        if start - 1 < jb < end + 1 and math.log(rng.uniform()) < lng[ib - 1] - lng[jb - 1]:
            acc += 1
            e = e_sw
        else:
            cfg[a[2], a[1], a[0]], cfg[b[2], b[1], b[0]] = s1, s2
            jb = ib
        if period > 0 and i % period == 0:
            hist[jb - start] += 1.0
            if store is not None and store["open"][jb - 1]:
                store["open"][jb - 1] = 0
                store["slots"][jb - 1] = cfg
        lng[jb - 1] += f
    return acc, e


def test_sweeps_with_neighbour_swaps_match_python_restatement():
    rng = np.random.default_rng(8)
    ns, nsh, n = 3, 2, 3
    V = np.zeros((ns, ns, nsh))
    for sh in range(nsh):
        a = rng.uniform(-0.05, 0.05, size=(ns, ns))
        V[:, :, sh] = (np.triu(a) + np.triu(a, 1).T) / 13.605693122
    mod = O.OracleModel("bcc", n, n, n, V)
    cfg, _ = mod.initial_setup(O.OracleRng(3), np.array([0.0, 1 / 3, 1 / 3, 1 / 3]), np.array([18, 18, 18]))
    e0 = mod.total_energy(cfg)
    bins = 60
    edges = (e0 - 0.02) + np.arange(bins + 1) * (0.04 / bins)
    start, end, n_trials, period = 10, 50, 4000, 1
    cfg_a, cfg_b = cfg.copy(), cfg.copy()
    lng_a, lng_b = np.zeros(bins), np.zeros(bins)
    hist_a, hist_b = np.zeros(end - start + 1), np.zeros(end - start + 1)
    ra, rb = O.OracleRng(77), O.OracleRng(77)
    acc_a, e_a, c = mod.wl_sweep(cfg_a, ra, edges, lng_a, hist_a, e0, bins, start, end, n_trials, 1.0, period,
                                 nbr_swap=True)
    acc_b, e_b = _py_sweeps_nbr(mod, n, cfg_b, rb, edges, lng_b, hist_b, e0, bins, start, end, n_trials,
                                1.0, period)
    assert acc_a == acc_b > 0
    assert e_a == e_b
    assert np.array_equal(cfg_a, cfg_b)
    assert np.array_equal(lng_a, lng_b) and np.array_equal(hist_a, hist_b)
    assert np.array_equal(ra.state_words(), rb.state_words())
    assert c.draws == 4 * n_trials + c.exp_tests


def _radial_state(bins, wc, ns, cap, done_every=0):
    done = np.zeros(bins, dtype=np.uint8)
    if done_every:
        done[::done_every] = 1
    return {"shells": None, "cap": cap, "done": done, "record": np.zeros(bins, dtype=np.int32),
            "rho_of_E": np.zeros((bins, wc, ns, ns)), "steps": np.zeros(1, dtype=np.int32)}


@pytest.mark.parametrize("nbr", [False, True])
def test_sweeps_radial_samples_match_python_restatement(nbr):
    """rho_of_E, radial_record and radial_mc_steps of sweeps() against the
    reference's lines written out, with some bins already complete
    (radial_record_bool) and a per-walker cap of 2 samples."""
    rng = np.random.default_rng(9)
    ns, nsh, n, wc = 3, 2, 3, 3
    V = np.zeros((ns, ns, nsh))
    for sh in range(nsh):
        a = rng.uniform(-0.05, 0.05, size=(ns, ns))
        V[:, :, sh] = (np.triu(a) + np.triu(a, 1).T) / 13.605693122
    mod = O.OracleModel("bcc", n, n, n, V)
    cfg, _ = mod.initial_setup(O.OracleRng(5), np.array([0.0, 1 / 3, 1 / 3, 1 / 3]), np.array([18, 18, 18]))
    shells = mod.lattice_shells(cfg, wc)
    e0 = mod.total_energy(cfg)
    bins = 40
    edges = (e0 - 0.03) + np.arange(bins + 1) * (0.06 / bins)
    start, end, n_trials, period = 5, 35, 6000, 1
    ra, rb = _radial_state(bins, wc, ns, 2, 7), _radial_state(bins, wc, ns, 2, 7)
    ra["shells"] = rb["shells"] = np.ascontiguousarray(shells)
    ra["steps"][0] = rb["steps"][0] = 17
    cfg_a, cfg_b = cfg.copy(), cfg.copy()
    lng_a, lng_b = np.zeros(bins), np.zeros(bins)
    hist_a, hist_b = np.zeros(end - start + 1), np.zeros(end - start + 1)
    ga, gb = O.OracleRng(31), O.OracleRng(31)
    acc_a, e_a, _ = mod.wl_sweep(cfg_a, ga, edges, lng_a, hist_a, e0, bins, start, end, n_trials, 1.0, period,
                                 nbr_swap=nbr, radial=ra)
    acc_b, e_b = _py_sweeps_nbr(mod, n, cfg_b, gb, edges, lng_b, hist_b, e0, bins, start, end, n_trials,
                                1.0, period, nbr=nbr, radial=rb)
    assert acc_a == acc_b and e_a == e_b and np.array_equal(cfg_a, cfg_b)
    assert np.array_equal(ra["record"], rb["record"]) and ra["record"].sum() > 3
    assert np.array_equal(ra["rho_of_E"], rb["rho_of_E"])
    assert ra["steps"][0] == rb["steps"][0]
    assert np.all(ra["record"][::7] == 0) and np.all(ra["record"] <= 2)


def _py_enter_window(mod, cfg, rng, conc, nums, min_e, max_e, sig2x2, max_steps):
    """enter_energy_window (src/wang-landau.F90:643-741) written out from the
    reference, one walker, the oracle giving sites, energies and
    initial_setup."""
    target = (min_e + max_e) / 2.0
    cond = abs(max_e - min_e) * 0.1
    reinit = mod.n_atoms * 50 * 5
    e_un = mod.total_energy(cfg)
    i_steps = 0
    for it in range(1, max_steps + 1):
        i_steps += 1
        if i_steps % reinit == 0:
            i_steps = 0
            new, _ = mod.initial_setup(rng, conc, nums)
            cfg[...] = new
        if max_e - cond > e_un > min_e + cond:
            e_un = mod.total_energy(cfg)
            if max_e - cond > e_un > min_e + cond:
                return it, e_un
            continue
        a, b = mod.random_site(rng), mod.random_site(rng)
        s1, s2 = cfg[a[2], a[1], a[0]], cfg[b[2], b[1], b[0]]
        if s1 != s2:
            p_un = mod.pair_energy(cfg, a, b)
            cfg[a[2], a[1], a[0]], cfg[b[2], b[1], b[0]] = s2, s1
            e_sw = e_un - p_un + mod.pair_energy(cfg, a, b)
            d = ((e_sw - target) * (e_sw - target) - (e_un - target) * (e_un - target)) / sig2x2
            if math.log(rng.uniform()) < -d:
                e_un = e_sw
            else:
                cfg[a[2], a[1], a[0]], cfg[b[2], b[1], b[0]] = s1, s2
    return -1, e_un


def test_enter_window_matches_python_restatement():
    rng = np.random.default_rng(13)
    ns, nsh, n = 3, 2, 3
    V = np.zeros((ns, ns, nsh))
    for sh in range(nsh):
        a = rng.uniform(-0.05, 0.05, size=(ns, ns))
        V[:, :, sh] = (np.triu(a) + np.triu(a, 1).T) / 13.605693122
    mod = O.OracleModel("bcc", n, n, n, V)
    conc = np.array([0.0, 1 / 3, 1 / 3, 1 / 3])
    nums = np.array([18, 18, 18])
    cfg, _ = mod.initial_setup(O.OracleRng(5), conc, nums)
    e0 = mod.total_energy(cfg)
    # a window below the start: the walk has to go down
    lo, hi = e0 - 0.04, e0 - 0.02
    sig2x2 = 2.0 * (float(np.float32(0.0025)) * 40.0 * 54 / (13.605693122 * 1000)) ** 2
    ca, cb = cfg.copy(), cfg.copy()
    ra, rb = O.OracleRng(91), O.OracleRng(91)
    it_a, e_a = mod.wl_enter_window(ca, ra, conc, nums, lo, hi, sig2x2, 200000)
    it_b, e_b = _py_enter_window(mod, cb, rb, conc, nums, lo, hi, sig2x2, 200000)
    assert it_a == it_b > 0 and e_a == e_b
    assert np.array_equal(ca, cb)
    assert np.array_equal(ra.state_words(), rb.state_words())
    assert lo + 0.1 * (hi - lo) < e_a < hi - 0.1 * (hi - lo)


def test_enter_window_redraws_like_the_reference():
    """An unreachable window: the walk redraws the configuration every
    n_atoms * 250 steps (the running energy kept stale, as the reference
    keeps it) and stops at max_steps."""
    rng = np.random.default_rng(14)
    ns, nsh, n = 3, 2, 3
    V = np.zeros((ns, ns, nsh))
    for sh in range(nsh):
        a = rng.uniform(-0.05, 0.05, size=(ns, ns))
        V[:, :, sh] = (np.triu(a) + np.triu(a, 1).T) / 13.605693122
    mod = O.OracleModel("bcc", n, n, n, V)
    conc = np.array([0.0, 1 / 3, 1 / 3, 1 / 3])
    cfg, _ = mod.initial_setup(O.OracleRng(6), conc, np.array([18, 18, 18]))
    lo, hi = -100.0, -99.0
    sig2x2 = 0.5
    ca, cb = cfg.copy(), cfg.copy()
    ra, rb = O.OracleRng(92), O.OracleRng(92)
    it_a, e_a = mod.wl_enter_window(ca, ra, conc, np.array([18, 18, 18]), lo, hi, sig2x2, 30000)
    it_b, e_b = _py_enter_window(mod, cb, rb, conc, np.array([18, 18, 18]), lo, hi, sig2x2, 30000)
    assert it_a == it_b == -1 and e_a == e_b
    assert np.array_equal(ca, cb) and np.array_equal(ra.state_words(), rb.state_words())


def test_sweeps_store_keeps_the_first_sampled_configuration_per_bin():
    """config_per_bin (src/wang-landau.F90:605-610): a bin closes at its
    first histogram tick, so the closed bins are exactly those with ticks,
    each slot holds a configuration of that bin's energy, and a second call
    leaves closed slots alone."""
    rng = np.random.default_rng(3)
    V = np.zeros((3, 3, 2))
    for sh in range(2):
        a = rng.uniform(-0.05, 0.05, (3, 3))
        V[:, :, sh] = (np.triu(a) + np.triu(a, 1).T) / 13.6
    mod = O.OracleModel("bcc", 4, 4, 4, V)
    r = O.OracleRng(5)
    cfg, _ = mod.initial_setup(r, np.array([0.0, 1 / 3, 1 / 3, 1 / 3]))
    E = mod.total_energy(cfg)
    bins = 40
    edges = E - 0.2 + np.arange(bins + 1) * (0.4 / bins)
    lng, hist = np.zeros(bins), np.zeros(bins)
    store = dict(slots=np.zeros((bins,) + cfg.shape, dtype=np.int8), open=np.ones(bins, dtype=np.uint8))
    _, E, _ = mod.wl_sweep(cfg, r, edges, lng, hist, E, bins, 1, bins, 3000, 1.0, 2, store=store)
    closed = np.nonzero(store["open"] == 0)[0]
    assert closed.size > 0 and np.array_equal(closed, np.nonzero(hist > 0)[0])
    for b in closed:
        assert O.wl_bin_index(mod.total_energy(store["slots"][b]), edges, bins) == b + 1
        assert np.array_equal(np.bincount(store["slots"][b].ravel(), minlength=4),
                              np.bincount(cfg.ravel(), minlength=4))
    before = store["slots"].copy()
    mod.wl_sweep(cfg, r, edges, lng, hist, E, bins, 1, bins, 3000, 1.0, 2, store=store)
    assert np.array_equal(store["slots"][closed], before[closed])
    assert np.array_equal(np.nonzero(store["open"] == 0)[0], np.nonzero(hist > 0)[0])


@pytest.mark.parametrize("nbr", [False, True])
def test_sweeps_store_matches_python_restatement(nbr):
    """The oracle's configuration store against the restatement above, over
    two calls (the second one finds bins closed by the first)."""
    rng = np.random.default_rng(81)
    ns, nsh, n = 3, 2, 3
    V = np.zeros((ns, ns, nsh))
    for sh in range(nsh):
        a = rng.uniform(-0.05, 0.05, size=(ns, ns))
        V[:, :, sh] = (np.triu(a) + np.triu(a, 1).T) / 13.605693122
    mod = O.OracleModel("bcc", n, n, n, V)
    cfg, _ = mod.initial_setup(O.OracleRng(5), np.array([0.0, 1 / 3, 1 / 3, 1 / 3]), np.array([18, 18, 18]))
    e0 = mod.total_energy(cfg)
    bins = 60
    edges = (e0 - 0.02) + np.arange(bins + 1) * (0.04 / bins)
    start, end, period = 10, 50, 3
    cfg_a, cfg_b = cfg.copy(), cfg.copy()
    lng_a, lng_b = np.zeros(bins), np.zeros(bins)
    hist_a, hist_b = np.zeros(end - start + 1), np.zeros(end - start + 1)
    st_a = dict(slots=np.zeros((bins,) + cfg.shape, dtype=np.int8), open=np.ones(bins, dtype=np.uint8))
    st_b = dict(slots=np.zeros((bins,) + cfg.shape, dtype=np.int8), open=np.ones(bins, dtype=np.uint8))
    ra, rb = O.OracleRng(99), O.OracleRng(99)
    e_a = e_b = e0
    for _ in range(2):
        acc_a, e_a, _ = mod.wl_sweep(cfg_a, ra, edges, lng_a, hist_a, e_a, bins, start, end, 1500, 0.5, period,
                                     nbr_swap=nbr, store=st_a)
        acc_b, e_b = _py_sweeps_nbr(mod, n, cfg_b, rb, edges, lng_b, hist_b, e_b, bins, start, end, 1500, 0.5,
                                    period, nbr=nbr, store=st_b)
        assert acc_a == acc_b and e_a == e_b
    assert np.array_equal(st_a["open"], st_b["open"]) and (st_a["open"] == 0).any()
    assert np.array_equal(st_a["slots"], st_b["slots"])
    assert np.array_equal(cfg_a, cfg_b) and np.array_equal(hist_a, hist_b)
