"""Host drivers of the Metropolis modes over the GPU chain.

simulated_annealing mirrors metropolis_simulated_annealing
(src/metropolis.F90:84-558): per
temperature, the optional burn-in, the sample at step 0, n_sweeps blocks of
n_sweep_steps swap trials on the device, and after each block the energy
(total_energy), the ASRO sample (radial_densities), the ALRO sample
(store_state, on the device) and the trajectory rows.
The per-temperature averages use the reference's arithmetic: E and E^2
accumulated in FP64 sample by sample, n_save_* = floor(real/real) in single
precision, C clamped at zero.  decorrelated_samples mirrors
metropolis_decorrelated_samples (:560-738).  simulated_annealing_ensemble
runs the MPI ranks' annealings as the chains of one batch and averages them
as comms_reduce_metropolis_results does (src/comms.F90:122-160).
"""
from __future__ import annotations

import numpy as np

from . import K_B_IN_RY, Batch, Chain


def _f32_floor_div(a: int, b: int) -> int:
    return int(np.floor(np.float32(a) / np.float32(b)))


def _block_end(m, i: int, n_sweeps: int, n_sweep_steps: int) -> int:
    """The last sweep of the device block starting at sweep i: the first
    sweep from i on after which ASRO or ALRO is sampled (those read the
    configuration on the host), else the temperature's last sweep."""
    j = i
    while j < n_sweeps:
        step_n = j * n_sweep_steps
        if m.calculate_asro and step_n % m.n_sample_steps_asro == 0:
            break
        if m.calculate_alro and step_n % m.n_sample_steps_alro == 0:
            break
        j += 1
    return j


def simulated_annealing(chain: Chain, metropolis, wc_range: int, record_configs: bool = True):
    """Runs the annealing on a chain whose configuration and stream are
    already set (initial_setup or a read configuration).  `metropolis` is a
    MetropolisParams (brawl_gb300.inputs).  Returns per-temperature arrays and
    the trajectory, with the keys the reference writes to its outputs."""
    m = metropolis
    ns = chain.setup.n_species
    n_atoms = chain.setup.n_atoms
    shells = chain.lattice_shells(wc_range)
    n_save_energy = _f32_floor_div(m.n_mc_steps, m.n_sample_steps)
    n_save_asro = _f32_floor_div(m.n_mc_steps, m.n_sample_steps_asro)
    n_save_alro = _f32_floor_div(m.n_mc_steps, m.n_sample_steps_alro) if m.calculate_alro else 1
    Ts = m.T_steps
    out = {
        "shells": shells,
        "temperature": np.zeros(Ts), "energies_of_T": np.zeros(Ts), "C_of_T": np.zeros(Ts),
        "acceptance_of_T": np.zeros(Ts), "rho_of_T": np.zeros((Ts, wc_range, ns, ns)),
        "traj_step": [], "traj_energy": [], "traj_asro": [],
        "initial_configs": [], "final_configs": [],
        "order_of_T": (np.zeros((Ts,) + chain.setup.grid_shape + (1, ns)) if m.calculate_alro else None),
    }
    asro = np.zeros((wc_range, ns, ns))
    for j in range(Ts):
        r_dens = np.zeros((wc_range, ns, ns))
        step_E = 0.0
        step_Esq = 0.0
        temp = m.T + float(j) * m.delta_T
        sim_temp = temp * K_B_IN_RY
        beta = 1.0 / sim_temp if sim_temp != 0.0 else float("inf")
        out["temperature"][j] = temp
        if m.calculate_alro:
            chain.alro_reset()
        burn = m.burn_in_start if j == 0 else m.burn_in
        if burn and m.n_burn_in_steps > 0:
            chain.metropolis(beta, m.n_burn_in_steps, m.nbr_swap)
        current_energy = 0.0
        if m.calculate_energies:
            current_energy = chain.total_energy()
        if m.calculate_asro:
            asro = chain.radial_densities(shells)
        out["traj_step"].append(0)
        out["traj_energy"].append(current_energy)
        out["traj_asro"].append(asro.copy())
        if record_configs:
            out["initial_configs"].append(chain.config())
        n_sweeps = m.n_mc_steps // m.n_sample_steps
        n_sweep_steps = m.n_mc_steps // n_sweeps
        accepted = 0
        block_E = None
        block_end = 0
        for i in range(1, n_sweeps + 1):
            if i > block_end:
                # the sweeps up to the next ASRO / ALRO sample run as one
                # device block, their energies sampled on the device
                block_end = _block_end(m, i, n_sweeps, n_sweep_steps)
                block_E, acc = chain.anneal_sweeps(beta, block_end - i + 1, n_sweep_steps, m.nbr_swap,
                                                   energies=bool(m.calculate_energies))
                block_first = i
                accepted += acc
            step_n = i * n_sweep_steps
            if m.calculate_energies:
                current_energy = float(block_E[i - block_first])
                step_E = step_E + current_energy
                step_Esq = step_Esq + current_energy * current_energy
            if m.calculate_asro and step_n % m.n_sample_steps_asro == 0:
                asro = chain.radial_densities(shells)
                r_dens = r_dens + asro
            if m.calculate_alro and step_n % m.n_sample_steps_alro == 0:
                chain.alro_add()
            if step_n % m.n_sample_steps_trajectory == 0:
                out["traj_step"].append(step_n)
                out["traj_energy"].append(current_energy)
                out["traj_asro"].append(asro.copy())
        # acceptance/real(n_mc_steps): the sum of 0/1 results is exact in FP64
        out["acceptance_of_T"][j] = float(accepted) / float(np.float32(m.n_mc_steps))
        if m.calculate_energies:
            ne = float(n_save_energy)
            out["energies_of_T"][j] = step_E / ne / float(n_atoms)
            mean = step_E / ne
            C = (step_Esq / ne - mean * mean) / (sim_temp * temp) / float(n_atoms)
            if C < 0.0:
                C = 0.0
            if temp <= 0.0:
                C = 0.0
            out["C_of_T"][j] = C
        if m.calculate_asro:
            out["rho_of_T"][j] = r_dens / float(n_save_asro)
        if m.calculate_alro:
            # order / real(n_save_alro): the count in single precision, exact
            out["order_of_T"][j] = chain.alro() / float(np.float32(n_save_alro))
        if record_configs:
            out["final_configs"].append(chain.config())
    out["traj_step"] = np.array(out["traj_step"], dtype=np.int64)
    out["traj_energy"] = np.array(out["traj_energy"])
    out["traj_asro"] = np.array(out["traj_asro"])
    return out


def decorrelated_samples(chain: Chain, metropolis, record_configs: bool = True):
    """metropolis_decorrelated_samples (src/metropolis.F90:560-738) on a
    chain whose configuration and stream are already set.  As the reference
    does it: the burn-in (when burn_in) runs at every temperature
    T + (j-1) delta_T in turn, then one sampling loop of n_mc_steps trials at
    the last temperature's beta, with a sample every n_sample_steps trials --
    the energy (full_energy) and the configuration (written as xyz by the
    reference) -- and the acceptance counter reset at each sample.  Returns
    the burn-in acceptances per temperature and the samples."""
    m = metropolis
    if m.T_steps < 1:
        raise ValueError("decorrelated_samples needs T_steps >= 1")
    temps = np.array([m.T + float(j) * m.delta_T for j in range(m.T_steps)])
    out = {"temperature": temps, "burn_in_accepted": np.zeros(m.T_steps, dtype=np.int64),
           "sample_step": [], "sample_energy": [], "sample_accepted": [], "configs": []}
    beta = float("inf")
    for j, temp in enumerate(temps):
        sim_temp = temp * K_B_IN_RY
        beta = 1.0 / sim_temp if sim_temp != 0.0 else float("inf")
        if m.burn_in and m.n_burn_in_steps > 0:
            out["burn_in_accepted"][j] = chain.metropolis(beta, m.n_burn_in_steps, m.nbr_swap)
    step = 0
    accepted = 0
    while step < m.n_mc_steps:
        # up to the next multiple of n_sample_steps (or the end of the loop)
        chunk = min(m.n_sample_steps - step % m.n_sample_steps, m.n_mc_steps - step)
        accepted += chain.metropolis(beta, chunk, m.nbr_swap)
        step += chunk
        if step % m.n_sample_steps == 0:
            out["sample_step"].append(step)
            out["sample_energy"].append(chain.total_energy())
            out["sample_accepted"].append(accepted)
            if record_configs:
                out["configs"].append(chain.config())
            accepted = 0
    out["sample_step"] = np.array(out["sample_step"], dtype=np.int64)
    out["sample_energy"] = np.array(out["sample_energy"])
    out["sample_accepted"] = np.array(out["sample_accepted"], dtype=np.int64)
    return out


def simulated_annealing_ensemble(batch: Batch, metropolis, wc_range: int, record_configs: bool = True):
    """metropolis_simulated_annealing on every chain of a batch at once (the
    reference's ranks, each with its own stream and configuration), every
    sweep block one launch for all chains.  Each chain's outputs are what
    simulated_annealing gives for it alone; "average" holds the ensemble
    averages of comms_reduce_metropolis_results: the rank sum in rank order
    divided by real(p).  The sampling reductions run on the device
    (brawl_batch_sampling_reset / energy_sample / asro_sample /
    temperature_stats / asro_stats): the E and E^2 sums, the radial-density
    sums, the per-temperature energies, heat capacities, acceptance rates and
    radial densities and their averages over the chains; the host only
    collects the trajectory rows and the results."""
    m = metropolis
    n = batch.n
    if any(b != bool(m.nbr_swap) for b in batch.nbr_swap):
        raise ValueError("the batch's chains must be created with nbr_swap = metropolis.nbr_swap")
    ns = batch.setups[0].n_species
    shells = [batch.lattice_shells(c, wc_range) for c in range(n)]
    n_save_energy = _f32_floor_div(m.n_mc_steps, m.n_sample_steps)
    n_save_asro = _f32_floor_div(m.n_mc_steps, m.n_sample_steps_asro)
    n_save_alro = _f32_floor_div(m.n_mc_steps, m.n_sample_steps_alro) if m.calculate_alro else 1
    Ts = m.T_steps
    outs = [{
        "shells": shells[c],
        "temperature": np.zeros(Ts), "energies_of_T": np.zeros(Ts), "C_of_T": np.zeros(Ts),
        "acceptance_of_T": np.zeros(Ts), "rho_of_T": np.zeros((Ts, wc_range, ns, ns)),
        "traj_step": [], "traj_energy": [], "traj_asro": [],
        "initial_configs": [], "final_configs": [],
        "order_of_T": (np.zeros((Ts,) + batch.setups[c].grid_shape + (1, ns)) if m.calculate_alro else None),
    } for c in range(n)]
    av = {"acceptance_of_T": np.zeros(Ts)}
    if m.calculate_energies:
        av["energies_of_T"] = np.zeros(Ts)
        av["C_of_T"] = np.zeros(Ts)
    if m.calculate_asro:
        av["rho_of_T"] = np.zeros((Ts, wc_range, ns, ns))
    asro = [np.zeros((wc_range, ns, ns)) for _ in range(n)]
    for j in range(Ts):
        temp = m.T + float(j) * m.delta_T
        sim_temp = temp * K_B_IN_RY
        beta = 1.0 / sim_temp if sim_temp != 0.0 else float("inf")
        batch.set_beta(np.full(n, beta))
        if m.calculate_alro:
            batch.alro_reset()
        burn = m.burn_in_start if j == 0 else m.burn_in
        if burn and m.n_burn_in_steps > 0:
            batch.metropolis(m.n_burn_in_steps)
        batch.sampling_reset(wc_range if m.calculate_asro else 0)
        energy = batch.total_energy() if m.calculate_energies else np.zeros(n)
        if m.calculate_asro:
            asro = [batch.radial_densities(c, shells[c]) for c in range(n)]
        for c in range(n):
            o = outs[c]
            o["temperature"][j] = temp
            o["traj_step"].append(0)
            o["traj_energy"].append(energy[c])
            o["traj_asro"].append(asro[c].copy())
            if record_configs:
                o["initial_configs"].append(batch.config(c))
        n_sweeps = m.n_mc_steps // m.n_sample_steps
        n_sweep_steps = m.n_mc_steps // n_sweeps
        block_E = None
        block_end = 0
        for i in range(1, n_sweeps + 1):
            if i > block_end:
                # the sweeps up to the next ASRO / ALRO sample run as one
                # device block, their energies sampled on the device
                block_end = _block_end(m, i, n_sweeps, n_sweep_steps)
                block_E, _ = batch.anneal_sweeps(block_end - i + 1, n_sweep_steps,
                                                 accumulate=bool(m.calculate_energies),
                                                 energies=bool(m.calculate_energies))
                block_first = i
            step_n = i * n_sweep_steps
            if m.calculate_energies:
                energy = block_E[i - block_first]
            if m.calculate_asro and step_n % m.n_sample_steps_asro == 0:
                asro = [batch.asro_sample(c, shells[c]) for c in range(n)]
            if m.calculate_alro and step_n % m.n_sample_steps_alro == 0:
                batch.alro_add()
            if step_n % m.n_sample_steps_trajectory == 0:
                for c in range(n):
                    outs[c]["traj_step"].append(step_n)
                    outs[c]["traj_energy"].append(energy[c])
                    outs[c]["traj_asro"].append(asro[c].copy())
        per, avT = batch.temperature_stats(n_save_energy if m.calculate_energies else 1, m.n_mc_steps,
                                           temp, sim_temp, bool(m.calculate_energies))
        av["acceptance_of_T"][j] = avT[2]
        if m.calculate_energies:
            av["energies_of_T"][j] = avT[0]
            av["C_of_T"][j] = avT[1]
        if m.calculate_asro:
            rho_c, rho_av = batch.asro_stats(n_save_asro)
            av["rho_of_T"][j] = rho_av
        for c in range(n):
            o = outs[c]
            o["acceptance_of_T"][j] = per[2][c]
            if m.calculate_energies:
                o["energies_of_T"][j] = per[0][c]
                o["C_of_T"][j] = per[1][c]
            if m.calculate_asro:
                o["rho_of_T"][j] = rho_c[c]
            if m.calculate_alro:
                o["order_of_T"][j] = batch.alro(c) / float(np.float32(n_save_alro))
            if record_configs:
                o["final_configs"].append(batch.config(c))
    for o in outs:
        o["traj_step"] = np.array(o["traj_step"], dtype=np.int64)
        o["traj_energy"] = np.array(o["traj_energy"])
        o["traj_asro"] = np.array(o["traj_asro"])
    return {"ranks": outs, "average": av}
