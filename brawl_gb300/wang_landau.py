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
(:757-808) is optional (pre_sample=True).  Left out: window optimisation
and the configuration reloads it needs, and the per-bin
configuration reloads (which draw from gfortran's random_number).  The
density of states is therefore the reference's only statistically (its own
test compares against the stored result with a 1% NRMSE criterion), which
is the comparison made here.
"""
from __future__ import annotations

import math

import numpy as np

from . import K_B_IN_RY, RY_TO_EV, Batch, Setup, WangLandauWalkers

__all__ = ["create_energy_bins", "divide_range", "create_overlap", "save_rho_E", "compute_mean_energy",
           "wang_landau"]


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
                 exchange: bool = True, max_calls: int = 1_000_000) -> int:
    """pre_sampling (src/wang-landau.F90:757-808) up to its dos_average and
    dos_combine: sweeps() of every walker at the initial wl_f, replica
    exchange after the 10th call and every 9th after it, until every
    window is pre-sampled -- a window is as soon as one of its walkers has
    min(hist) > 1000/num_walkers and is flatter than wl_flatness (the
    reference's MPI_MAX over ranks); a walker of a pre-sampled window has its
    histogram set to n_atoms + 1 once.  Returns the sweeps() calls made."""
    trials = wl.mc_sweeps * n_atoms
    period = int(0.02 * float(np.float32(n_atoms)))
    nwin = wl.num_windows
    done = np.zeros(nwin, dtype=bool)
    state = np.zeros(W.n, dtype=bool)
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
        flat = W.flatness()
        for k in range(W.n):
            if not state[k] and flat[k] > wl.flatness and W.hist(k).min() > 1000.0 / float(walkers_per_window):
                done[k // walkers_per_window] = True
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
                burn_in: str = "temperature", numbers=None, pre_sample: bool = False) -> dict:
    """Runs the main loop to wl.tolerance.  wl: the wl_input fields
    (mc_sweeps, bins, num_windows, bin_overlap, tolerance, flatness, wl_f,
    energy_min, energy_max).  radial (optional): dict(wc_range, shells,
    radial_samples) turns on the radial-density samples.  Returns the
    combined ln g, the bin edges, the windows, the iteration record and,
    with radial samples, rho_of_E once every bin has its samples."""
    n_atoms = setup.n_atoms
    edges = create_energy_bins(n_atoms, wl.energy_min, wl.energy_max, wl.bins)
    windows = create_overlap(divide_range(wl.bins, wl.num_windows), wl.bin_overlap)
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
    trials = wl.mc_sweeps * n_atoms
    period = int(0.02 * float(np.float32(n_atoms)))
    pre_calls = 0
    if pre_sample:
        pre_calls = pre_sampling(W, wl, walkers_per_window, n_atoms, f, exchange, max_calls)
        W.reset_hist()                   # mpi_wl_hist = 0 before the main loop
    converged = np.zeros(n, dtype=bool)
    record = []
    calls = 0
    lng = np.zeros(wl.bins)
    while f > wl.tolerance and calls < max_calls:
        W.sweeps(trials, f, period)
        calls += 1
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
            record.append({"calls": calls, "wl_f": f})
            if log:
                log(f"ln f -> {f:.3e} after {calls} sweeps() calls")
    if radial is not None:
        save_rho_E(W, radial["radial_samples"], rad_state)
    W.close()
    mean_energy = compute_mean_energy(lng, edges, wl.bins,
                                      bin_width_ry(n_atoms, wl.energy_min, wl.energy_max, wl.bins))
    return {"lng": lng, "bin_edges": edges, "windows": windows, "record": record, "calls": calls,
            "rho_of_E": rad_state["rho_of_E"], "radial_min": rad_state["radial_min"],
            "burn_in_steps": burn_steps, "mean_energy": mean_energy, "pre_sampling_calls": pre_calls}
