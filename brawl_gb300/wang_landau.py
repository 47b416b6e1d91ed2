"""The Wang-Landau driver (src/wang-landau.F90, wl_main) over the device
walkers of brawl_gb300.WangLandauWalkers.

Kept as the reference has them: the energy bins (create_energy_bins,
:969-992), the windows and their overlaps (divide_range :855-891,
create_overlap :934-955), the main loop (:198-300) -- sweeps() of every
walker, replica exchange between adjacent windows, per-walker flatness with
the converged flag held until every walker is flat, then ln f halved, the
histograms reset, dos_average and dos_combine -- until ln f falls below the
tolerance -- and, when asked, the radial-density samples of sweeps() with
save_rho_E's bookkeeping (:359-396).  The burn-in into the windows is the
reference's enter_energy_window (:643-741) on the device (burn_in =
"reference"): the biased walk of every walker from initial_setup on its own
stream; of the walkers of a window, the one that got in first (fewest
iterations, then the lowest index, where the reference's MPI race decides)
hands its configuration to the others.  Alternatively (burn_in =
"temperature") a temperature search with the device Metropolis kernel that
stops each walker inside the same central 80% of its window.  Pre-sampling
(:757-808) is optional (pre_sample=True); with it come the per-bin
configuration store of sweeps() (config_per_bin, kept on the device),
merge_configs and load_window_config (:1541-1615), and the window
optimisation mpi_window_optimise (:1211-1328) as wl_input's performance
setting asks for it.  The reference draws the merge's and the reloads'
choices from gfortran's random_number, and MPI timing decides its
burn-in's hand-over; here they come from numpy's generator and from the
walkers' iteration counts.  The density of states is therefore the
reference's only statistically (its own test compares against the stored
result with a 1% NRMSE criterion), which is the comparison made here.
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import K_B_IN_RY, RY_TO_EV, Batch, Setup, WangLandauWalkers

__all__ = ["create_energy_bins", "divide_range", "create_overlap", "save_rho_E", "compute_mean_energy",
           "window_optimise", "sort_descending", "merge_configs", "load_window_config", "wang_landau"]


def bin_width_ry(n_atoms: int, energy_min: float, energy_max: float, bins: int) -> float:
    """bin_width (src/wang-landau.F90:976-980): energy_min/max are default
    (single precision) reals, so (energy_max - energy_min)/real(bins) is
    single precision; the conversion to Ry, n_atoms/(Ry_to_eV*1000), double."""
    f32 = np.float32
    w = f32(f32(f32(energy_max) - f32(energy_min)) / f32(bins))
    return float(w) * (n_atoms / (RY_TO_EV * 1000.0))


def create_energy_bins(n_atoms: int, energy_min: float, energy_max: float, bins: int) -> np.ndarray:
    """bin_edges(1:bins+1) in Ry from meV/atom (src/wang-landau.F90:969-992)."""
    energy_to_ry = n_atoms / (RY_TO_EV * 1000.0)
    bin_width = bin_width_ry(n_atoms, energy_min, energy_max, bins)
    e0 = float(np.float32(energy_min)) * energy_to_ry
    return np.array([e0 + i * bin_width for i in range(bins + 1)])


def divide_range(bins: int, num_windows: int) -> list[list[int]]:
    """window_intervals: 1-based [first, last] bin of every window (power 1)."""
    w = [[0, 0] for _ in range(num_windows)]
    w[0][0] = 1
    w[-1][1] = bins
    factor = (bins - 1.0) / ((num_windows + 1.0) ** 1 - 1.0)
    for i in range(2, num_windows + 1):
        w[i - 2][1] = int(math.floor(factor * ((i - 1) ** 1) + 1))
        w[i - 1][0] = w[i - 2][1] + 1
    return w


def create_overlap(intervals: list[list[int]], bin_overlap: float) -> list[list[int]]:
    """window_indices: every window but the first extended downwards by
    max(ceiling(bin_overlap * previous window's bins), 2) (the last window
    counts the previous one's bins without the +1, as the reference does)."""
    n = len(intervals)
    idx = [list(x) for x in intervals]
    if n > 1:
        for i in range(2, n):
            b = idx[i - 2][1] - idx[i - 2][0] + 1
            idx[i - 1][0] = int(intervals[i - 1][0] - max(math.ceil(bin_overlap * b), 2))
            idx[i - 1][1] = intervals[i - 1][1]
        b = idx[n - 2][1] - idx[n - 2][0]
        idx[n - 1][0] = int(intervals[n - 1][0] - max(math.ceil(bin_overlap * b), 2))
        idx[n - 1][1] = intervals[n - 1][1]
    return idx


def _burn_in(setup: Setup, V, seeds, conc, targets, n_atoms, max_rounds=400):
    """Configurations with energies inside (lo, hi) for every walker, from
    initial_setup followed by Metropolis runs whose temperature is raised
    when the energy is below the target and lowered when above."""
    n = len(seeds)
    T = np.full(n, 3000.0)
    chains = [dict(setup=setup, V=V, seed=int(s), beta=1.0 / (3000.0 * K_B_IN_RY), species_concentrations=conc)
              for s in seeds]
    b = Batch(chains)
    done = np.zeros(n, dtype=bool)
    cfgs = [None] * n
    E = b.total_energy()
    for _ in range(max_rounds):
        for k in range(n):
            lo, hi = targets[k]
            if not done[k] and lo < E[k] < hi:
                done[k] = True
                cfgs[k] = b.config(k)
        if done.all():
            break
        for k in range(n):
            if done[k]:
                continue
            lo, hi = targets[k]
            T[k] = T[k] * (0.8 if E[k] > hi else 1.25)
        b.set_beta(1.0 / (T * K_B_IN_RY))
        trials = np.where(done, 0, 10 * n_atoms).astype(np.int64)
        b.metropolis(trials)
        E = b.total_energy()
    if not done.all():
        raise RuntimeError("burn-in did not reach every window")
    rng_states = [b.rng_state(k) for k in range(n)]
    b.close()
    return cfgs, rng_states


def _seq_sum(a: np.ndarray) -> float:
    """SUM as a left-to-right loop."""
    return float(np.cumsum(a)[-1]) if a.size else 0.0


def _powi(x: float, n: int) -> float:
    """real ** integer as gfortran evaluates it: binary exponentiation
    (libgcc's __powidf2), not pow()."""
    m = abs(n)
    y = x if m % 2 else 1.0
    m >>= 1
    while m:
        x = x * x
        if m % 2:
            y = y * x
        m >>= 1
    return 1.0 / y if n < 0 else y


def _nint(x: float) -> int:
    """NINT: the nearest integer, halves away from zero."""
    a = abs(x)
    f = math.floor(a)
    r = int(f) + (1 if a - f >= 0.5 else 0)
    return r if x >= 0 else -r


def sort_descending(a) -> list[int]:
    """sort_descending (src/wang-landau.F90:1686-1703): the exchange sort of
    the index list by a descending (0-based here)."""
    n = len(a)
    idx = list(range(n))
    for i in range(n - 1):
        for j in range(i + 1, n):
            if a[idx[i]] < a[idx[j]]:
                idx[i], idx[j] = idx[j], idx[i]
    return idx


def window_optimise(iteration: int, intervals, wl_mc_steps, diffusion_prev, bins: int,
                    performance: int = 0, max_cycles: int = 1_000_000):
    """mpi_window_optimise (src/wang-landau.F90:1211-1328) on rank 0: the
    windows resized from the MC steps each took to converge (wl_mc_steps,
    summed over its walkers), mixed with the previous fractions
    (diffusion_prev) by alpha = 0.8 * 0.8**(iteration-1), or 1 for iteration
    0; every window keeps at least max(INT(0.02 bins), 2) bins, and rounding
    is settled over the windows by descending size.  The per-window bin
    count is taken, as in the reference, as ABS(first - last + 1).  Returns
    (intervals, diffusion_prev), both new; unchanged for one window or a
    performance setting outside 0-3.  The ln g weights the reference also
    computes do not enter the result and are left out."""
    nwin = len(intervals)
    old = [list(x) for x in intervals]
    prev = np.array(diffusion_prev, dtype=np.float64)
    if performance not in (0, 1, 2, 3) or nwin <= 1:
        return old, prev
    alpha = 0.8 * _powi(0.8, iteration - 1)
    if iteration == 0:
        alpha = 1.0
    w_min = 0.02
    steps = np.asarray(wl_mc_steps, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        weights_mc = np.array([np.float64(1.0) / (steps[i] / np.float64(abs(old[i][0] - old[i][1] + 1)))
                               for i in range(nwin)])
        weights_mc = weights_mc / _seq_sum(weights_mc)
        frac = alpha * weights_mc + (1.0 - alpha) * prev
        frac = frac / _seq_sum(frac)
    diffusion_new = frac.copy()
    frac = np.maximum(frac, w_min)
    free = frac > w_min
    if abs(_seq_sum(frac) - 1.0) > 1.0e-12:
        rem = 1.0 - _seq_sum(frac)
        if free.any():
            sum_free = 0.0
            for i in range(nwin):
                if free[i]:
                    sum_free = sum_free + frac[i]
            if sum_free > 0.0:
                scale = rem / sum_free
                for i in range(nwin):
                    if free[i]:
                        frac[i] = frac[i] + frac[i] * scale
    frac = frac / _seq_sum(frac)
    nb = [_nint(float(np.float32(bins)) * float(frac[i])) for i in range(nwin)]
    min_bins = max(int(w_min * bins), 2)
    nb = [max(x, min_bins) for x in nb]
    if sum(nb) != bins:
        idx = sort_descending(nb)
        diff = bins - sum(nb)
        i = 1
        while diff != 0:
            if i > max_cycles * nwin:  # the reference loops for ever here
                raise RuntimeError("window_optimise: cannot shrink the windows to the bin count")
            j = idx[(i - 1) % nwin]
            if diff > 0:
                nb[j] += 1
                diff -= 1
            elif diff < 0 and nb[j] > min_bins:
                nb[j] -= 1
                diff += 1
            i += 1
    new = [list(x) for x in old]
    new[0][1] = nb[0]
    for i in range(1, nwin):
        new[i][0] = new[i - 1][1] + 1
        new[i][1] = new[i][0] + nb[i] - 1
    new[nwin - 1][0] = new[nwin - 2][1] + 1
    new[nwin - 1][1] = bins
    return new, diffusion_new


def merge_configs(W: WangLandauWalkers, rng: np.random.Generator) -> np.ndarray:
    """merge_configs (src/wang-landau.F90:1556-1615): for every bin, one
    walker among those holding a configuration for it, drawn uniformly, and
    every walker's slot becomes that one (the bin reopens where none holds
    it).  The draws come from rng where the reference calls gfortran's
    random_number.  Returns the picks (-1: none)."""
    open_ = W.store_flags()
    pick = np.full(W.bins, -1, dtype=np.int32)
    for b in range(W.bins):
        holders = np.nonzero(~open_[:, b])[0]
        if holders.size:
            pick[b] = int(holders[int(rng.random() * holders.size)])
    W.store_merge(pick)
    return pick


def load_window_config(W: WangLandauWalkers, windows, walkers_per_window: int,
                       rng: np.random.Generator) -> np.ndarray:
    """load_window_config (src/wang-landau.F90:1541-1554) on every walker:
    a bin of its window (overlap included) drawn uniformly, and the stored
    configuration of that bin.  Returns the bins drawn."""
    out = np.zeros(W.n, dtype=np.int64)
    for k in range(W.n):
        s, e = windows[k // walkers_per_window]
        b = s + int(rng.random() * float(e - s + 1))
        W.store_load(k, b)
        out[k] = b
    return out


def compute_mean_energy(lng, bin_edges, bins: int, bin_width: float) -> np.ndarray:
    """compute_mean_energy (src/wang-landau.F90:457-477): for T = 10, 20,
    ..., 3000 K, the canonical mean energy from ln g over the bin centres.
    Returns mean_energy(itemp, 1:2) as (300, 2): the mean energy and beta.
    The exponentials use numpy's exp, which may differ from the C library's
    in the last bit, so the values are the reference's to rounding."""
    buf = np.asarray(lng, dtype=np.float64) - np.max(lng)
    centres = np.asarray(bin_edges[:bins], dtype=np.float64) + 0.5 * bin_width
    out = np.zeros((300, 2))
    for itemp in range(1, 301):
        beta = 1.0 / (K_B_IN_RY * itemp * 10.0)
        prob = buf - beta * centres
        prob = np.exp(prob - np.max(prob))
        prob = prob / _seq_sum(prob)
        out[itemp - 1, 0] = _seq_sum(centres * prob)
        out[itemp - 1, 1] = beta
    return out


def pre_sampling(W: WangLandauWalkers, wl, walkers_per_window: int, n_atoms: int, f: float,
                 exchange: bool = True, max_calls: int = 1_000_000, mc_steps: np.ndarray | None = None) -> int:
    """pre_sampling (src/wang-landau.F90:757-808) up to its dos_average and
    dos_combine: sweeps() of every walker at the initial wl_f, replica
    exchange after the 10th call and every 9th after it, until every
    window is pre-sampled -- a window is as soon as one of its walkers has
    min(hist) > 1000/num_walkers and is flatter than wl_flatness (the
    reference's MPI_MAX over ranks); a walker of a pre-sampled window has its
    histogram set to n_atoms + 1 once.  mc_steps (optional, per window)
    gets wl_mc_steps: every walker's trials until its own criterion held
    (:774-776).  Returns the sweeps() calls made."""
    trials = wl.mc_sweeps * n_atoms
    period = int(0.02 * float(np.float32(n_atoms)))
    nwin = wl.num_windows
    done = np.zeros(nwin, dtype=bool)
    state = np.zeros(W.n, dtype=bool)
    own = np.zeros(W.n, dtype=bool)      # pre_sampled(mpi_index) of each rank
    i_sweeps = 0
    calls = 0
    while not done.all() and calls < max_calls:
        W.sweeps(trials, f, period)
        calls += 1
        i_sweeps += 1
        if i_sweeps % 10 == 0:
            i_sweeps = 1
            if exchange and nwin > 1:
                W.replica_exchange()
        if mc_steps is not None:
            for k in range(W.n):
                if not own[k]:
                    mc_steps[k // walkers_per_window] += float(trials)
        flat = W.flatness()
        for k in range(W.n):
            if not state[k] and flat[k] > wl.flatness and W.hist(k).min() > 1000.0 / float(walkers_per_window):
                done[k // walkers_per_window] = True
                own[k] = True
        for k in range(W.n):
            if done[k // walkers_per_window] and not state[k]:
                state[k] = True
                h = W.hist(k)
                W.set_hist(k, np.full(h.size, float(np.float32(n_atoms)) + 1.0))
    W.average()
    W.dos_combine()
    return calls


def save_rho_E(W: WangLandauWalkers, radial_samples: int, state: dict) -> None:
    """save_rho_E (src/wang-landau.F90:359-396): the walkers' radial_record
    summed (walker order for the reference's MPI_REDUCE), radial_record_bool
    set where the sum reaches radial_samples, and once every bin is set the
    walkers' rho_of_E summed and divided by the bin's count (rho_saved)."""
    if state["rho_saved"]:
        return
    recs, rhos = [], []
    for w in range(W.n):
        r, rho, _ = W.radial(w)
        recs.append(r)
        rhos.append(rho)
    total = recs[0].astype(np.int64)
    for r in recs[1:]:
        total = total + r
    done = total >= radial_samples
    W.radial_set_done(done)
    state["radial_min"] = float(np.float32(np.count_nonzero(done)) / np.float32(done.size))
    if done.all():
        state["rho_saved"] = True
        s = rhos[0].copy()
        for rho in rhos[1:]:
            s = s + rho
        counts = total.astype(np.float32).astype(np.float64)
        state["rho_of_E"] = s / counts[:, None, None, None]


def wang_landau(setup: Setup, V, conc, wl, walkers_per_window: int = 1, seed0: int = 110179,
                exchange: bool = True, max_calls: int = 1_000_000, log=None, radial=None,
                burn_in: str = "temperature", numbers=None, pre_sample: bool = False,
                config_store: bool | None = None, optimise_windows: bool | None = None,
                store_seed: int = 0, trials_per_call: int | None = None,
                deadline_s: float | None = None) -> dict:
    """Runs the main loop to wl.tolerance.  wl: the wl_input fields
    (mc_sweeps, bins, num_windows, bin_overlap, tolerance, flatness, wl_f,
    energy_min, energy_max, performance).  radial (optional): dict(wc_range,
    shells, radial_samples) turns on the radial-density samples.

    config_store (default: pre_sample) keeps config_per_bin on the device:
    pre-sampling then ends with merge_configs and load_window_config, and
    every ln f step with load_window_config, as the reference's do.
    Pre-sampling is what makes every bin of every window stored; without it
    a reload can draw a bin no walker has visited, which raises BrawlError
    (the reference would load its zero-filled slot).
    optimise_windows (default: config_store) resizes the windows with
    mpi_window_optimise where wl.performance asks for it (0-3 after
    pre-sampling, 0-1 at every ln f step); it needs the store, which gives
    the walkers configurations inside their new windows.  The draws the
    reference takes from gfortran's random_number come from numpy's
    generator seeded with store_seed.

    trials_per_call (default mc_sweeps * n_atoms) sets the trials of every
    sweeps() call, i.e. the replica-exchange interval.  deadline_s stops the
    main loop after that many seconds (wall clock) like max_calls does.

    Returns the combined ln g, the bin edges, the windows (the last ones)
    and every set used, the iteration record and, with radial samples,
    rho_of_E once every bin has its samples."""
    n_atoms = setup.n_atoms
    edges = create_energy_bins(n_atoms, wl.energy_min, wl.energy_max, wl.bins)
    intervals = divide_range(wl.bins, wl.num_windows)
    windows = create_overlap(intervals, wl.bin_overlap)
    store = bool(pre_sample) if config_store is None else bool(config_store)
    optimise = store if optimise_windows is None else bool(optimise_windows)
    if optimise and not store:
        raise ValueError("optimise_windows needs config_store")
    performance = int(getattr(wl, "performance", 0))
    host_rng = np.random.default_rng(store_seed)
    window_sets = [[list(x) for x in windows]]
    n = wl.num_windows * walkers_per_window
    seeds = [seed0 + 11 * r for r in range(n)]
    targets = []
    for r in range(n):
        s, e = windows[r // walkers_per_window]
        lo_e, hi_e = edges[s - 1], edges[e]
        cond = abs(hi_e - lo_e) * 0.1
        targets.append((lo_e + cond, hi_e - cond))
    if burn_in == "temperature":
        cfgs, _ = _burn_in(setup, V, seeds, conc, targets, n_atoms)
    elif burn_in == "reference":
        # placeholders: enter_windows draws every walker's start with initial_setup
        tmp = Batch([dict(setup=setup, V=V, seed=seeds[0], beta=0.0, species_concentrations=conc,
                          species_numbers=numbers)])
        cfgs = [tmp.config(0)] * n
        tmp.close()
    else:
        raise ValueError(f"unknown burn_in {burn_in!r}")
    walkers = [dict(setup=setup, V=V, seed=seeds[r], config=cfgs[r], start_idx=windows[r // walkers_per_window][0],
                    end_idx=windows[r // walkers_per_window][1], window=r // walkers_per_window,
                    nbr_swap=bool(getattr(wl, "nbr_swap", False))) for r in range(n)]
    W = WangLandauWalkers(walkers, edges)
    if store:
        W.store_enable()                 # config_per_bin = 0, config_store = .True.
    burn_steps = None
    if burn_in == "reference":
        burn_steps = W.enter_windows(wl.energy_min, wl.energy_max, conc, numbers, initial=True)
        for win in range(wl.num_windows):
            ks = list(range(win * walkers_per_window, (win + 1) * walkers_per_window))
            first = min(ks, key=lambda k: (burn_steps[k], k))
            for k in ks:
                if k != first:
                    W.set_config(k, W.config(first))
    rad_state = {"rho_saved": True, "rho_of_E": None, "radial_min": 0.0}
    if radial is not None:
        W.radial_enable(radial["wc_range"], radial["shells"], radial["radial_samples"], walkers_per_window)
        rad_state["rho_saved"] = False
    f = float(wl.wl_f)
    trials = wl.mc_sweeps * n_atoms if trials_per_call is None else int(trials_per_call)
    period = int(0.02 * float(np.float32(n_atoms)))
    pre_calls = 0
    nwin = wl.num_windows
    mc_steps = np.zeros(nwin)            # wl_mc_steps, summed over each window's walkers
    diffusion_prev = np.full(nwin, 1.0 / float(nwin))

    def new_windows(iteration: int) -> None:
        nonlocal intervals, windows, diffusion_prev
        intervals, diffusion_prev = window_optimise(iteration, intervals, mc_steps, diffusion_prev, wl.bins,
                                                    performance)
        windows = create_overlap(intervals, wl.bin_overlap)
        W.set_windows([w[0] for w in windows], [w[1] for w in windows])
        window_sets.append([list(x) for x in windows])

    if pre_sample:
        pre_calls = pre_sampling(W, wl, walkers_per_window, n_atoms, f, exchange, max_calls, mc_steps)
        if optimise and nwin > 1 and performance in (0, 1, 2, 3):
            new_windows(0)               # mpi_window_optimise(0) (:820)
        mc_steps[:] = 0.0
        if store:
            merge_configs(W, host_rng)
            load_window_config(W, windows, walkers_per_window, host_rng)
        W.reset_hist()                   # mpi_wl_hist = 0 before the main loop
    it = 2                               # iter after pre-sampling (:176, :190)
    converged = np.zeros(n, dtype=bool)
    record = []
    calls = 0
    lng = np.zeros(wl.bins)
    t_start = time.perf_counter()
    while f > wl.tolerance and calls < max_calls:
        if deadline_s is not None and time.perf_counter() - t_start > deadline_s:
            break
        W.sweeps(trials, f, period)
        calls += 1
        for k in range(n):
            if not converged[k]:         # wl_mc_steps until the walker's flatness (:216-218)
                mc_steps[k // walkers_per_window] += float(trials)
        if exchange and wl.num_windows > 1:
            W.replica_exchange()
        flat = W.flatness()
        converged |= flat > wl.flatness
        if converged.all():
            converged[:] = False
            W.reset_hist()
            f *= 0.5
            W.average()
            lng = W.dos_combine()
            if radial is not None:
                save_rho_E(W, radial["radial_samples"], rad_state)
            if optimise and nwin > 1 and performance in (0, 1):
                new_windows(it - 1)      # mpi_window_optimise(iter-1) (:284-286)
            mc_steps[:] = 0.0
            if store:
                load_window_config(W, windows, walkers_per_window, host_rng)
            it += 1
            record.append({"calls": calls, "wl_f": f, "seconds": time.perf_counter() - t_start})
            if log:
                log(f"ln f -> {f:.3e} after {calls} sweeps() calls")
    if radial is not None:
        save_rho_E(W, radial["radial_samples"], rad_state)
    W.close()
    mean_energy = compute_mean_energy(lng, edges, wl.bins,
                                      bin_width_ry(n_atoms, wl.energy_min, wl.energy_max, wl.bins))
    return {"lng": lng, "bin_edges": edges, "windows": windows, "window_sets": window_sets,
            "record": record, "calls": calls,
            "rho_of_E": rad_state["rho_of_E"], "radial_min": rad_state["radial_min"],
            "burn_in_steps": burn_steps, "mean_energy": mean_energy, "pre_sampling_calls": pre_calls}
