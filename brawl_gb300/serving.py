"""Serving: the continuous-batching request loop of include/brawl_gpu.h
(brawl_serve_*) and the job stream it is measured on.

Jobs are anneals (the reference's metropolis_simulated_annealing with one
energy sample per temperature, src/metropolis.F90:84-558), Wang-Landau
windows (sweeps() with in-window averaging and ln f halving on flatness,
src/wang-landau.F90:539-632) and nested-sampling runs
(src/nested_sampling.f90:45-206).  Each job is a dict; `Server.submit`
queues it and the library's scheduler thread admits it by device memory and
slot count and runs it in shared launches with every other resident job.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

# The server keeps long rounds of kernels in flight on a few streams while
# jobs are set up and read back on their own; with the default 8 hardware
# work queues those would often share a queue with a round and wait for it.
# Takes effect if this module is imported before the CUDA context exists.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

from . import BrawlError, K_B_IN_RY, LATTICES, RY_TO_EV, Setup, _Setup, _check, _ptr, _v_array, load

KINDS = {"anneal": 1, "wl": 2, "ns": 3}
KIND_NAMES = {v: k for k, v in KINDS.items()}
EAGAIN, ETIMEDOUT = 7, 4


class _Opts(C.Structure):
    _fields_ = [("hbm_budget", C.c_size_t), ("max_active", C.c_int), ("round_ms", C.c_double),
                ("max_trials", C.c_int64), ("max_iterations", C.c_int), ("max_active_wl", C.c_int),
                ("max_active_ns", C.c_int)]


class _JobDesc(C.Structure):
    _fields_ = [("kind", C.c_int), ("setup", _Setup), ("V_ex", C.c_void_p), ("seed", C.c_uint32),
                ("species_concentrations", C.c_void_p), ("species_numbers", C.c_void_p),
                ("T_start", C.c_double), ("delta_T", C.c_double), ("T_steps", C.c_int),
                ("sweeps_per_T", C.c_int64),
                ("wl_walkers", C.c_int), ("wl_bins", C.c_int), ("wl_calls", C.c_int),
                ("wl_trials", C.c_int64),
                ("wl_half_width", C.c_double), ("wl_f", C.c_double), ("wl_flatness", C.c_double),
                ("wl_tolerance", C.c_double),
                ("ns_walkers", C.c_int), ("ns_steps", C.c_int), ("ns_iter", C.c_int)]


class _JobResult(C.Structure):
    _fields_ = [("status", C.c_int), ("kind", C.c_int), ("t_submit", C.c_double),
                ("t_admit", C.c_double), ("t_finish", C.c_double), ("t_ready", C.c_double),
                ("trials", C.c_int64),
                ("accepted", C.c_int64), ("energy", C.c_double), ("wl_f", C.c_double),
                ("wl_halvings", C.c_int), ("n_values", C.c_int)]


def _result_dict(r: _JobResult) -> dict:
    return {k: getattr(r, k) for k, _ in _JobResult._fields_}


class Server:
    """A brawl_server: submit jobs, wait for them, read their values."""

    def __init__(self, hbm_budget: int = 0, max_active: int = 0, round_ms: float = 0.0,
                 max_trials: int = 0, max_iterations: int = 0, max_active_wl: int = 0,
                 max_active_ns: int = 0):
        o = _Opts(hbm_budget, max_active, round_ms, max_trials, max_iterations, max_active_wl, max_active_ns)
        h = C.c_void_p()
        _check(load().brawl_serve_create(C.byref(o), C.byref(h)))
        self._h = h
        self._setups: dict[int, Setup] = {}

    def close(self):
        if getattr(self, "_h", None):
            load().brawl_serve_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, job: dict) -> int:
        s: Setup = job["setup"]
        V = _v_array(s, job["V"])
        conc = np.ascontiguousarray(job["conc"], dtype=np.float64)
        if conc.size != s.n_species + 1:
            raise ValueError("conc needs n_species+1 entries ([0] = 0)")
        numbers = job.get("numbers")
        nums = None if numbers is None else np.ascontiguousarray(numbers, dtype=np.int64)
        d = _JobDesc()
        d.kind = KINDS[job["kind"]]
        d.setup = s.c()
        d.V_ex = V.ctypes.data
        d.seed = int(job["seed"]) & 0xFFFFFFFF
        d.species_concentrations = conc.ctypes.data
        d.species_numbers = None if nums is None else nums.ctypes.data
        for k in ("T_start", "delta_T", "wl_half_width", "wl_f", "wl_flatness", "wl_tolerance"):
            setattr(d, k, float(job.get(k, 0.0)))
        for k in ("T_steps", "sweeps_per_T", "wl_walkers", "wl_bins", "wl_calls", "wl_trials",
                  "ns_walkers", "ns_steps", "ns_iter"):
            setattr(d, k, int(job.get(k, 0)))
        jid = C.c_uint64()
        _check(load().brawl_serve_submit(self._h, C.byref(d), C.byref(jid)))
        self._setups[jid.value] = s
        return jid.value

    def poll(self, jid: int) -> dict | None:
        r = _JobResult()
        rc = load().brawl_serve_poll(self._h, jid, C.byref(r))
        if rc == EAGAIN:
            return None
        _check(rc)
        return _result_dict(r)

    def wait(self, jid: int, timeout: float | None = None) -> dict:
        r = _JobResult()
        _check(load().brawl_serve_wait(self._h, jid, -1.0 if timeout is None else float(timeout),
                                       C.byref(r)))
        return _result_dict(r)

    def values(self, jid: int, n_values: int) -> np.ndarray:
        out = np.zeros(max(n_values, 1), dtype=np.float64)
        _check(load().brawl_serve_values(self._h, jid, _ptr(out)))
        return out[:n_values]

    def config(self, jid: int) -> np.ndarray:
        out = np.zeros(self._setups[jid].grid_shape, dtype=np.int8)
        _check(load().brawl_serve_config(self._h, jid, _ptr(out)))
        return out

    def release(self, jid: int) -> None:
        _check(load().brawl_serve_release(self._h, jid))
        self._setups.pop(jid, None)

    def profile(self) -> dict:
        """Per pipeline: rounds, device-busy, launch and settle seconds, work
        handed out (trials; Wang-Landau summed over walkers; nested sampling
        walk steps at n_steps per iteration)."""
        v = np.zeros(15)
        _check(load().brawl_serve_profile(self._h, _ptr(v)))
        return {k: {"rounds": int(v[5 * i]), "busy_s": v[5 * i + 1], "launch_s": v[5 * i + 2],
                    "settle_s": v[5 * i + 3], "work": int(v[5 * i + 4])}
                for i, k in enumerate(("anneal", "wl", "ns"))}

    def stats(self) -> dict:
        s = np.zeros(4, dtype=np.int64)
        _check(load().brawl_serve_stats(self._h, _ptr(s)))
        return {"rounds": int(s[0]), "resident": int(s[1]), "queued": int(s[2]), "ended": int(s[3])}


def symmetric_V(rng: np.random.Generator, ns: int, nsh: int, half_ev: float) -> np.ndarray:
    """V(s,s',shell) symmetric in the species, uniform [-half, half] eV, in Ry."""
    V = np.zeros((ns, ns, nsh))
    for sh in range(nsh):
        a = rng.uniform(-half_ev, half_ev, (ns, ns))
        V[:, :, sh] = np.triu(a) + np.triu(a, 1).T
    return V / RY_TO_EV


def n_sites(lattice: str, L: int) -> int:
    return {"fcc": 4, "bcc": 2, "sc": 8}[lattice] * L ** 3


def stream_jobs(n_jobs: int, master_seed: int = 424242, L_range=(6, 32), sweeps_range=(100, 2000)):
    """The seeded mixed job stream: lattice in {fcc, bcc}, L in L_range,
    2-5 species with a Dirichlet(1) composition rounded to counts, 2-6
    shells, V uniform [-0.05, 0.05] eV; kind anneal (sweeps in
    sweeps_range, one temperature band of 4 steps), a Wang-Landau window
    (4 walkers, 256 bins over E0 -/+ 5 meV/atom, 20 calls of one sweep) or a nested-sampling run
    (64 walkers, one-sweep walks, 100 iterations).  Every job carries its
    own seed drawn from the master seed."""
    rng = np.random.default_rng(master_seed)
    jobs = []
    for k in range(n_jobs):
        lattice = "fcc" if rng.integers(2) == 0 else "bcc"
        L = int(rng.integers(L_range[0], L_range[1] + 1))
        ns = int(rng.integers(2, 6))
        nsh = int(rng.integers(2, 7))
        N = n_sites(lattice, L)
        w = rng.dirichlet(np.ones(ns))
        counts = np.floor(w * N).astype(np.int64)
        counts = np.maximum(counts, 1)
        while counts.sum() < N:
            counts[int(np.argmax(w * N - counts))] += 1
        while counts.sum() > N:
            counts[int(np.argmax(counts))] -= 1
        conc = np.concatenate([[0.0], counts / N])
        V = symmetric_V(rng, ns, nsh, 0.05)
        kind = ["anneal", "wl", "ns"][int(rng.integers(3))]
        job = {"kind": kind, "setup": Setup(lattice, L, L, L, ns, nsh), "V": V,
               "seed": int(rng.integers(1, 2 ** 31)), "conc": conc, "numbers": counts,
               "lattice": lattice, "L": L, "N": N}
        if kind == "anneal":
            sweeps = int(rng.integers(sweeps_range[0], sweeps_range[1] + 1))
            T0 = float(rng.uniform(300.0, 3000.0))
            job.update(T_start=T0, delta_T=-T0 / 8.0, T_steps=4, sweeps_per_T=max(sweeps // 4, 1))
        elif kind == "wl":
            job.update(wl_walkers=4, wl_bins=256, wl_calls=20, wl_trials=N,
                       wl_half_width=N * 5.0e-3 / RY_TO_EV, wl_f=1.0, wl_flatness=0.8,
                       wl_tolerance=1e-6)
        else:
            job.update(ns_walkers=64, ns_steps=N, ns_iter=100)
        jobs.append(job)
    return jobs


def job_trials(job: dict) -> int:
    """Swap trials the job performs (NS: walk steps at least)."""
    N = job["N"]
    if job["kind"] == "anneal":
        return job["T_steps"] * job["sweeps_per_T"] * N
    if job["kind"] == "wl":
        return job["wl_walkers"] * job["wl_calls"] * job["wl_trials"]
    return job["ns_iter"] * job["ns_steps"]
