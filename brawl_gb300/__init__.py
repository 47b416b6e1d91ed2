"""brawl_gb300 -- GB300 (sm_103a) implementation of BraWl's lattice-sampling
hot path, reached through the C ABI of include/brawl_gpu.h.

The Python layer here is host logic only: it mirrors the reference's
operator interface (total_energy, pair_energy, monte_carlo_step runs,
initial_setup, radial_densities, the annealing driver) over the CUDA library
libbrawl_gpu.so built in-tree by brawl_gb300.build.  There is no CPU
fallback: every call fails loudly when the library or a GPU is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

__all__ = ["load", "Setup", "Chain", "Batch", "NestedSampling", "WangLandauWalkers", "BrawlError",
           "LATTICES",
           "K_B_IN_RY", "RY_TO_EV"]

# src/constants.f90:41-49 (as written there)
K_B_IN_EV = 8.167333262e-5
K_B_IN_RY = 8.167333262e-5 / 13.605693122990
RY_TO_EV = 13.605693122

LATTICES = {"simple_cubic": 0, "sc": 0, "bcc": 1, "fcc": 2}
NUM_COUNTERS = 8
COUNTER_NAMES = ("trials", "evaluated", "draws", "accepted", "exp_tests", "exact_path",
                 "exp_fp64", "exp_cr")


class BrawlError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"brawl error {code}: {msg}")
        self.code = code


class _Setup(C.Structure):
    _fields_ = [("lattice", C.c_int), ("n_1", C.c_int), ("n_2", C.c_int), ("n_3", C.c_int),
                ("n_species", C.c_int), ("interaction_range", C.c_int)]


class _NsDesc(C.Structure):
    _fields_ = [("setup", _Setup), ("V_ex", C.c_void_p), ("seed", C.c_uint32),
                ("n_walkers", C.c_int), ("n_steps", C.c_int),
                ("species_concentrations", C.c_void_p), ("species_numbers", C.c_void_p)]


class _WlDesc(C.Structure):
    _fields_ = [("setup", _Setup), ("V_ex", C.c_void_p), ("seed", C.c_uint32),
                ("config", C.c_void_p), ("start_idx", C.c_int), ("end_idx", C.c_int),
                ("window", C.c_int), ("nbr_swap", C.c_int)]


class _ChainDesc(C.Structure):
    _fields_ = [("setup", _Setup), ("V_ex", C.c_void_p), ("seed", C.c_uint32),
                ("beta", C.c_double), ("nbr_swap", C.c_int),
                ("species_concentrations", C.c_void_p), ("species_numbers", C.c_void_p),
                ("config", C.c_void_p)]


_LIB = None


def load(rebuild: bool = False):
    """The CUDA library, built if needed.  Raises when it cannot be loaded."""
    global _LIB
    if _LIB is not None and not rebuild:
        return _LIB
    path = _build.LIB
    if rebuild or not os.path.exists(path):
        _build.build(force=rebuild)
    L = C.CDLL(path)
    vp, i, i64, d, u32 = C.c_void_p, C.c_int, C.c_int64, C.c_double, C.c_uint32
    sig = {
        "brawl_last_error": ([], C.c_char_p),
        "brawl_version": ([], i),
        "brawl_ctx_create": ([vp, vp, vp], i),
        "brawl_ctx_destroy": ([vp], i),
        "brawl_set_interactions": ([vp, vp], i),
        "brawl_seed": ([vp, u32], i),
        "brawl_f90_init_genrand": ([vp, i, i, u32, vp], i),
        "brawl_rng_get": ([vp, vp], i),
        "brawl_rng_set": ([vp, vp], i),
        "brawl_genrand": ([vp, i64, vp], i),
        "brawl_set_config": ([vp, vp], i),
        "brawl_get_config": ([vp, vp], i),
        "brawl_initial_setup": ([vp, vp, vp], i),
        "brawl_total_energy": ([vp, vp], i),
        "brawl_site_energy": ([vp, vp, vp], i),
        "brawl_pair_energy": ([vp, vp, vp, vp], i),
        "brawl_metropolis_run": ([vp, d, i64, i, vp], i),
        "brawl_anneal_sweeps": ([vp, d, i64, i64, i, vp, vp], i),
        "brawl_lattice_shells": ([vp, i, vp], i),
        "brawl_radial_densities": ([vp, i, vp, vp], i),
        "brawl_counters": ([vp, vp], i),
        "brawl_alro_add": ([vp], i),
        "brawl_alro_get": ([vp, vp], i),
        "brawl_alro_reset": ([vp], i),
        "brawl_total_energy_noalloc": ([vp, vp, vp, vp, vp], i),
        "brawl_ns_create": ([vp, i, vp], i),
        "brawl_ns_destroy": ([vp], i),
        "brawl_ns_iterate": ([vp, i, vp], i),
        "brawl_ns_energies": ([vp, i, vp], i),
        "brawl_ns_walker_config": ([vp, i, i, vp], i),
        "brawl_ns_counters": ([vp, i, vp], i),
        "brawl_wl_create": ([vp, i, i, vp, vp], i),
        "brawl_wl_destroy": ([vp], i),
        "brawl_wl_sweeps": ([vp, i64, d, i, vp], i),
        "brawl_wl_average": ([vp], i),
        "brawl_wl_get_lng": ([vp, i, vp], i),
        "brawl_wl_set_lng": ([vp, i, vp], i),
        "brawl_wl_get_hist": ([vp, i, vp], i),
        "brawl_wl_set_hist": ([vp, i, vp], i),
        "brawl_wl_energies": ([vp, vp], i),
        "brawl_wl_get_config": ([vp, i, vp], i),
        "brawl_wl_set_config": ([vp, i, vp], i),
        "brawl_wl_swap_configs": ([vp, i, i], i),
        "brawl_wl_genrand": ([vp, i, i64, vp], i),
        "brawl_wl_counters": ([vp, i, vp], i),
        "brawl_wl_radial_enable": ([vp, i, vp, i, i], i),
        "brawl_wl_enter_windows": ([vp, C.c_double, C.c_double, vp, vp, i, C.c_int64, vp], i),
        "brawl_wl_radial_set_done": ([vp, vp], i),
        "brawl_wl_radial_get": ([vp, i, vp, vp, vp], i),
        "brawl_wl_store_enable": ([vp], i),
        "brawl_wl_store_flags": ([vp, vp], i),
        "brawl_wl_store_merge": ([vp, vp], i),
        "brawl_wl_store_load": ([vp, i, i], i),
        "brawl_wl_store_get": ([vp, i, i, vp], i),
        "brawl_wl_set_windows": ([vp, vp, vp], i),
        "brawl_wl_replica_exchange": ([vp, vp, vp, vp], i),
        "brawl_wl_flatness": ([vp, vp], i),
        "brawl_wl_dos_combine": ([vp, vp], i),
        "brawl_wl_reset_hist": ([vp], i),
        "brawl_serve_create": ([vp, vp], i),
        "brawl_serve_destroy": ([vp], i),
        "brawl_serve_submit": ([vp, vp, vp], i),
        "brawl_serve_poll": ([vp, C.c_uint64, vp], i),
        "brawl_serve_wait": ([vp, C.c_uint64, d, vp], i),
        "brawl_serve_values": ([vp, C.c_uint64, vp], i),
        "brawl_serve_config": ([vp, C.c_uint64, vp], i),
        "brawl_serve_release": ([vp, C.c_uint64], i),
        "brawl_serve_stats": ([vp, vp], i),
        "brawl_serve_profile": ([vp, vp], i),
        "brawl_batch_create": ([vp, i, vp], i),
        "brawl_batch_destroy": ([vp], i),
        "brawl_batch_size": ([vp, vp], i),
        "brawl_batch_set_beta": ([vp, vp], i),
        "brawl_batch_set_speculation": ([vp, i], i),
        "brawl_batch_autotune": ([vp, vp, i, vp, vp], i),
        "brawl_batch_metropolis_run": ([vp, vp, vp], i),
        "brawl_batch_metropolis_run_async": ([vp, vp, vp], i),
        "brawl_batch_sync": ([vp], i),
        "brawl_batch_metropolis_run_serial": ([vp, vp, vp], i),
        "brawl_batch_total_energy": ([vp, vp], i),
        "brawl_batch_get_config": ([vp, i, vp], i),
        "brawl_batch_set_config": ([vp, i, vp], i),
        "brawl_batch_rng_get": ([vp, i, vp], i),
        "brawl_batch_get_configs": ([vp, vp], i),
        "brawl_batch_set_configs": ([vp, vp], i),
        "brawl_batch_metropolis_host": ([vp, vp, vp, vp, vp], i),
        "brawl_batch_counters": ([vp, vp], i),
        "brawl_batch_alro_add": ([vp], i),
        "brawl_batch_lattice_shells": ([vp, i, i, vp], i),
        "brawl_batch_alro_get": ([vp, i, vp], i),
        "brawl_batch_alro_reset": ([vp], i),
        "brawl_batch_radial_densities": ([vp, i, i, vp, vp], i),
        "brawl_batch_sampling_reset": ([vp, i], i),
        "brawl_batch_energy_sample": ([vp, vp], i),
        "brawl_batch_anneal_sweeps": ([vp, i64, i64, i, vp, vp], i),
        "brawl_batch_asro_sample": ([vp, i, vp, vp], i),
        "brawl_batch_temperature_stats": ([vp, i64, i64, d, d, i, vp, vp], i),
        "brawl_batch_asro_stats": ([vp, i64, vp, vp], i),
        "brawl_smem_bandwidth": ([vp], i),
        "brawl_batch_autotune_classes": ([vp, vp, i, vp, vp, vp], i),
        "brawl_batch_chain_classes": ([vp, vp], i),
        "brawl_batch_set_class_depths": ([vp, vp], i),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _LIB = L
    return L


def _check(rc: int) -> None:
    if rc != 0:
        raise BrawlError(rc, load().brawl_last_error().decode(errors="replace"))


def _ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


class Setup:
    """The subset of run_params (src/derived_types.f90:56-100) the path uses."""

    def __init__(self, lattice, n_1, n_2, n_3, n_species, interaction_range):
        self.lattice = LATTICES[lattice] if isinstance(lattice, str) else int(lattice)
        self.n = (int(n_1), int(n_2), int(n_3))
        self.n_species = int(n_species)
        self.interaction_range = int(interaction_range)

    @classmethod
    def from_run_params(cls, p) -> "Setup":
        return cls(p.lattice, p.n_1, p.n_2, p.n_3, p.n_species, p.interaction_range)

    def c(self) -> _Setup:
        return _Setup(self.lattice, *self.n, self.n_species, self.interaction_range)

    @property
    def grid_shape(self):
        """(z, y, x): the C-ordered view of config(1, 2n1, 2n2, 2n3)."""
        n1, n2, n3 = self.n
        return (2 * n3, 2 * n2, 2 * n1)

    @property
    def n_atoms(self) -> int:
        return (8, 2, 4)[self.lattice] * self.n[0] * self.n[1] * self.n[2]


def _v_array(setup: Setup, V) -> np.ndarray:
    V = np.asarray(V, dtype=np.float64)
    shape = (setup.n_species, setup.n_species, setup.interaction_range)
    if V.shape != shape:
        raise ValueError(f"V_ex must have shape {shape}, got {V.shape}")
    return np.ascontiguousarray(V.ravel(order="F"))


class Chain:
    """One simulation chain on the GPU (brawl_ctx): the reference's
    single-process state (config, V_ex, the mt19937ar stream)."""

    def __init__(self, setup: Setup, V):
        self.setup = setup
        self._V = _v_array(setup, V)
        h = C.c_void_p()
        s = setup.c()
        _check(load().brawl_ctx_create(C.byref(s), _ptr(self._V), C.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            load().brawl_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- generator ----------------------------------------------------------
    def seed(self, seed: int) -> None:
        _check(load().brawl_seed(self._h, seed))

    def f90_init_genrand(self, seedtime: int, my_rank: int, job_id: int = 0) -> int:
        out = C.c_uint32()
        _check(load().brawl_f90_init_genrand(self._h, seedtime, my_rank, job_id, C.byref(out)))
        return out.value

    def rng_state(self) -> np.ndarray:
        st = np.zeros(625, dtype=np.uint32)
        _check(load().brawl_rng_get(self._h, _ptr(st)))
        return st

    def set_rng_state(self, st) -> None:
        st = np.ascontiguousarray(st, dtype=np.uint32)
        _check(load().brawl_rng_set(self._h, _ptr(st)))

    def genrand(self, n: int) -> np.ndarray:
        out = np.zeros(n, dtype=np.float64)
        _check(load().brawl_genrand(self._h, n, _ptr(out)))
        return out

    # -- configuration -------------------------------------------------------
    def set_config(self, cfg: np.ndarray) -> None:
        cfg = np.ascontiguousarray(cfg, dtype=np.int8)
        if cfg.shape != self.setup.grid_shape:
            raise ValueError(f"config must have shape {self.setup.grid_shape}")
        _check(load().brawl_set_config(self._h, _ptr(cfg)))

    def config(self) -> np.ndarray:
        out = np.zeros(self.setup.grid_shape, dtype=np.int8)
        _check(load().brawl_get_config(self._h, _ptr(out)))
        return out

    def initial_setup(self, species_concentrations, species_numbers=None) -> np.ndarray:
        conc = np.ascontiguousarray(species_concentrations, dtype=np.float64).copy()
        if conc.shape != (self.setup.n_species + 1,):
            raise ValueError("species_concentrations needs n_species+1 entries ([0] = 0)")
        nums = None
        if species_numbers is not None:
            nums = np.ascontiguousarray(species_numbers, dtype=np.int64)
        _check(load().brawl_initial_setup(self._h, _ptr(conc), None if nums is None else _ptr(nums)))
        return conc

    # -- energies -------------------------------------------------------------
    def total_energy(self) -> float:
        e = C.c_double()
        _check(load().brawl_total_energy(self._h, C.byref(e)))
        return e.value

    def site_energy(self, idx) -> float:
        a = np.ascontiguousarray(idx, dtype=np.int32)
        e = C.c_double()
        _check(load().brawl_site_energy(self._h, _ptr(a), C.byref(e)))
        return e.value

    def pair_energy(self, idx1, idx2) -> float:
        a = np.ascontiguousarray(idx1, dtype=np.int32)
        b = np.ascontiguousarray(idx2, dtype=np.int32)
        e = C.c_double()
        _check(load().brawl_pair_energy(self._h, _ptr(a), _ptr(b), C.byref(e)))
        return e.value

    # -- sampling ---------------------------------------------------------------
    def metropolis(self, beta: float, n_trials: int, nbr_swap: bool = False) -> int:
        acc = C.c_int64()
        _check(load().brawl_metropolis_run(self._h, float(beta), int(n_trials), int(bool(nbr_swap)),
                                           C.byref(acc)))
        return acc.value

    def anneal_sweeps(self, beta: float, n_sweeps: int, sweep_trials: int, nbr_swap: bool = False,
                      energies: bool = True):
        """n_sweeps blocks of sweep_trials trials, the total energy after
        each block (the annealing loop's samples); returns (energies or
        None, accepted moves)."""
        out = np.zeros(int(n_sweeps), dtype=np.float64) if energies else None
        acc = C.c_int64()
        _check(load().brawl_anneal_sweeps(self._h, float(beta), int(n_sweeps), int(sweep_trials),
                                          int(bool(nbr_swap)), None if out is None else _ptr(out),
                                          C.byref(acc)))
        return out, acc.value

    def counters(self) -> dict:
        c = np.zeros(NUM_COUNTERS, dtype=np.int64)
        _check(load().brawl_counters(self._h, _ptr(c)))
        return dict(zip(COUNTER_NAMES, (int(v) for v in c)))

    # -- ALRO (store_state, src/analytics.f90:43-64) ----------------------------
    def alro_add(self) -> None:
        _check(load().brawl_alro_add(self._h))

    def alro_reset(self) -> None:
        _check(load().brawl_alro_reset(self._h))

    def alro(self) -> np.ndarray:
        """order(species, basis, x, y, z) as its C view, shaped
        (2n3, 2n2, 2n1, 1, n_species)."""
        out = np.zeros(self.setup.grid_shape + (1, self.setup.n_species), dtype=np.float64)
        _check(load().brawl_alro_get(self._h, _ptr(out)))
        return out

    # -- analytics ------------------------------------------------------------
    def lattice_shells(self, wc_range: int) -> np.ndarray:
        out = np.zeros(wc_range, dtype=np.float64)
        _check(load().brawl_lattice_shells(self._h, wc_range, _ptr(out)))
        return out

    def radial_densities(self, shells) -> np.ndarray:
        """rho shaped (wc_range, n_species, n_species): the C view of the
        reference's rho(i, j, l)."""
        shells = np.ascontiguousarray(shells, dtype=np.float64)
        wc = shells.shape[0]
        ns = self.setup.n_species
        out = np.zeros((wc, ns, ns), dtype=np.float64)
        _check(load().brawl_radial_densities(self._h, wc, _ptr(shells), _ptr(out)))
        return out


class Batch:
    """Many independent chains (brawl_batch) that run in one launch."""

    def __init__(self, chains: list[dict]):
        """Each chain: dict(setup=Setup, V=array, seed=int, beta=float,
        nbr_swap=bool, species_concentrations=array | None,
        species_numbers=array | None, config=array | None)."""
        n = len(chains)
        descs = (_ChainDesc * n)()
        self._keep = []
        self.setups = []
        self.nbr_swap = []
        for k, ch in enumerate(chains):
            s = ch["setup"]
            self.setups.append(s)
            self.nbr_swap.append(bool(ch.get("nbr_swap", False)))
            V = _v_array(s, ch["V"])
            self._keep.append(V)
            d = descs[k]
            d.setup = s.c()
            d.V_ex = V.ctypes.data
            d.seed = int(ch.get("seed", 5489)) & 0xFFFFFFFF
            d.beta = float(ch.get("beta", 0.0))
            d.nbr_swap = int(bool(ch.get("nbr_swap", False)))
            conc = ch.get("species_concentrations")
            if conc is not None:
                conc = np.ascontiguousarray(conc, dtype=np.float64)
                self._keep.append(conc)
                d.species_concentrations = conc.ctypes.data
            nums = ch.get("species_numbers")
            if nums is not None:
                nums = np.ascontiguousarray(nums, dtype=np.int64)
                self._keep.append(nums)
                d.species_numbers = nums.ctypes.data
            cfg = ch.get("config")
            if cfg is not None:
                cfg = np.ascontiguousarray(cfg, dtype=np.int8)
                self._keep.append(cfg)
                d.config = cfg.ctypes.data
        h = C.c_void_p()
        _check(load().brawl_batch_create(descs, n, C.byref(h)))
        self._h = h
        self.n = n
        self._keep = []

    def close(self):
        if getattr(self, "_h", None):
            load().brawl_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_beta(self, beta) -> None:
        b = np.ascontiguousarray(np.broadcast_to(np.asarray(beta, dtype=np.float64), (self.n,)))
        _check(load().brawl_batch_set_beta(self._h, _ptr(b)))

    def set_speculation(self, trials_per_round: int) -> None:
        """Trials per speculative round of the fcc/bcc kernel (1-4); speed only."""
        _check(load().brawl_batch_set_speculation(self._h, int(trials_per_round)))

    def autotune(self, n_trials, max_depth: int = 4) -> tuple[int, np.ndarray]:
        """Times n_trials of every chain at each trials-per-round depth
        1..max_depth from the same state (restored after each) and keeps
        the fastest; returns (depth, milliseconds per depth)."""
        t = self._trials(n_trials)
        ms = np.zeros(int(max_depth), dtype=np.float64)
        chosen = C.c_int()
        _check(load().brawl_batch_autotune(self._h, _ptr(t), int(max_depth), _ptr(ms), C.byref(chosen)))
        return chosen.value, ms

    def autotune_classes(self, n_trials, max_depth: int = 4) -> dict:
        """Trials per round picked per class of shared-memory chains (see
        brawl_batch_autotune_classes); returns per class its chains'
        lattice, L, species, shells, chain count, depth and ms per depth."""
        t = self._trials(n_trials)
        cls = np.zeros(self.n, dtype=np.int32)
        _check(load().brawl_batch_chain_classes(self._h, _ptr(cls)))
        nk = int(cls.max()) + 1 if (cls >= 0).any() else 0
        depths = np.zeros(max(nk, 1), dtype=np.int32)
        ms = np.zeros(max(nk, 1) * int(max_depth), dtype=np.float64)
        n = C.c_int()
        _check(load().brawl_batch_autotune_classes(self._h, _ptr(t), int(max_depth), _ptr(depths), _ptr(ms),
                                                   C.byref(n)))
        out = []
        for k in range(n.value):
            c = int(np.nonzero(cls == k)[0][0])
            s = self.setups[c]
            out.append({"lattice": {0: "sc", 1: "bcc", 2: "fcc"}[s.lattice], "L": list(s.n),
                        "species": s.n_species, "shells": s.interaction_range,
                        "chains": int((cls == k).sum()), "trials_per_round": int(depths[k]),
                        "ms_per_depth": [round(float(x), 2) for x in ms[k * max_depth:(k + 1) * max_depth]]})
        return {"classes": out}

    def chain_classes(self) -> np.ndarray:
        cls = np.zeros(self.n, dtype=np.int32)
        _check(load().brawl_batch_chain_classes(self._h, _ptr(cls)))
        return cls

    def set_class_depths(self, depths) -> None:
        d = np.ascontiguousarray(depths, dtype=np.int32)
        _check(load().brawl_batch_set_class_depths(self._h, _ptr(d)))

    def _trials(self, n_trials) -> np.ndarray:
        return np.ascontiguousarray(np.broadcast_to(np.asarray(n_trials, dtype=np.int64), (self.n,)))

    def metropolis(self, n_trials) -> np.ndarray:
        t = self._trials(n_trials)
        acc = np.zeros(self.n, dtype=np.int64)
        _check(load().brawl_batch_metropolis_run(self._h, _ptr(t), _ptr(acc)))
        return acc

    def metropolis_async(self, n_trials, stream: int | None = None) -> None:
        self._pending = self._trials(n_trials)
        _check(load().brawl_batch_metropolis_run_async(self._h, _ptr(self._pending),
                                                       C.c_void_p(stream) if stream else None))

    def sync(self) -> None:
        _check(load().brawl_batch_sync(self._h))

    def metropolis_serial(self, n_trials) -> np.ndarray:
        t = self._trials(n_trials)
        acc = np.zeros(self.n, dtype=np.int64)
        _check(load().brawl_batch_metropolis_run_serial(self._h, _ptr(t), _ptr(acc)))
        return acc

    def total_energy(self) -> np.ndarray:
        out = np.zeros(self.n, dtype=np.float64)
        _check(load().brawl_batch_total_energy(self._h, _ptr(out)))
        return out

    def config(self, c: int) -> np.ndarray:
        out = np.zeros(self.setups[c].grid_shape, dtype=np.int8)
        _check(load().brawl_batch_get_config(self._h, c, _ptr(out)))
        return out

    def set_config(self, c: int, cfg) -> None:
        cfg = np.ascontiguousarray(cfg, dtype=np.int8)
        _check(load().brawl_batch_set_config(self._h, c, _ptr(cfg)))

    def rng_state(self, c: int) -> np.ndarray:
        st = np.zeros(625, dtype=np.uint32)
        _check(load().brawl_batch_rng_get(self._h, c, _ptr(st)))
        return st

    @property
    def grid_bytes(self) -> int:
        return sum(int(np.prod(s.grid_shape)) for s in self.setups)

    def get_configs(self, out: np.ndarray | None = None) -> np.ndarray:
        """All chains' grids concatenated (int8, grid_bytes)."""
        if out is None:
            out = np.zeros(self.grid_bytes, dtype=np.int8)
        assert out.dtype == np.int8 and out.size == self.grid_bytes and out.flags.c_contiguous
        _check(load().brawl_batch_get_configs(self._h, _ptr(out)))
        return out

    def set_configs(self, grids: np.ndarray) -> None:
        assert grids.dtype == np.int8 and grids.size == self.grid_bytes and grids.flags.c_contiguous
        _check(load().brawl_batch_set_configs(self._h, _ptr(grids)))

    def metropolis_host(self, grids_in: np.ndarray, n_trials, grids_out: np.ndarray | None = None) -> np.ndarray:
        """set_configs + metropolis + get_configs in one call from host
        buffers (page-locked ones are used in place by the kernels);
        grids_out defaults to grids_in.  Returns the accepted moves."""
        if grids_out is None:
            grids_out = grids_in
        for g in (grids_in, grids_out):
            assert g.dtype == np.int8 and g.size == self.grid_bytes and g.flags.c_contiguous
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(n_trials, dtype=np.int64), (self.n,)))
        acc = np.zeros(self.n, dtype=np.int64)
        _check(load().brawl_batch_metropolis_host(self._h, _ptr(grids_in), _ptr(t), _ptr(grids_out), _ptr(acc)))
        return acc

    def counters(self) -> np.ndarray:
        out = np.zeros((self.n, NUM_COUNTERS), dtype=np.int64)
        _check(load().brawl_batch_counters(self._h, _ptr(out)))
        return out

    def radial_densities(self, c: int, shells) -> np.ndarray:
        shells = np.ascontiguousarray(shells, dtype=np.float64)
        wc = shells.shape[0]
        ns = self.setups[c].n_species
        out = np.zeros((wc, ns, ns), dtype=np.float64)
        _check(load().brawl_batch_radial_densities(self._h, c, wc, _ptr(shells), _ptr(out)))
        return out

    def lattice_shells(self, c: int, wc_range: int) -> np.ndarray:
        out = np.zeros(wc_range, dtype=np.float64)
        _check(load().brawl_batch_lattice_shells(self._h, c, wc_range, _ptr(out)))
        return out

    # -- sampling sums of the annealing loop, on the device ---------------------
    def sampling_reset(self, wc_range: int = 0) -> None:
        """Zero every chain's E, E^2 (and, wc_range >= 1, radial-density)
        sums and note the accepted counts: the start of a sampling loop."""
        self._samp_wc = int(wc_range)
        _check(load().brawl_batch_sampling_reset(self._h, int(wc_range)))

    def energy_sample(self, energies: bool = True) -> np.ndarray | None:
        """Every chain's total_energy added to its sums; returns them."""
        out = np.zeros(self.n, dtype=np.float64) if energies else None
        _check(load().brawl_batch_energy_sample(self._h, None if out is None else _ptr(out)))
        return out

    def anneal_sweeps(self, n_sweeps: int, sweep_trials: int, accumulate: bool = False,
                      energies: bool = True):
        """n_sweeps blocks of sweep_trials trials on every chain, each
        chain's total energy after every block (added to the sampling sums
        with accumulate); returns (energies[n_sweeps, n] or None, accepted
        moves per chain)."""
        out = np.zeros((int(n_sweeps), self.n), dtype=np.float64) if energies else None
        acc = np.zeros(self.n, dtype=np.int64)
        _check(load().brawl_batch_anneal_sweeps(self._h, int(n_sweeps), int(sweep_trials), int(bool(accumulate)),
                                                None if out is None else _ptr(out), _ptr(acc)))
        return out, acc

    def asro_sample(self, c: int, shells, rho: bool = True) -> np.ndarray | None:
        """Chain c's radial_densities added to its sums; returns them."""
        shells = np.ascontiguousarray(shells, dtype=np.float64)
        ns = self.setups[c].n_species
        out = np.zeros((shells.shape[0], ns, ns), dtype=np.float64) if rho else None
        _check(load().brawl_batch_asro_sample(self._h, c, _ptr(shells), None if out is None else _ptr(out)))
        return out

    def temperature_stats(self, n_save_energy: int, n_mc_steps: int, temp: float, sim_temp: float,
                          with_energies: bool = True):
        """(per-chain energies_of_T, C_of_T, acceptance_of_T; their averages
        over the chains), formed on the device."""
        per = np.zeros(3 * self.n, dtype=np.float64)
        av = np.zeros(3, dtype=np.float64)
        _check(load().brawl_batch_temperature_stats(self._h, int(n_save_energy), int(n_mc_steps), float(temp),
                                                    float(sim_temp), int(bool(with_energies)), _ptr(per),
                                                    _ptr(av)))
        return per.reshape(3, self.n), av

    def asro_stats(self, n_save_asro: int):
        """(per-chain rho_of_T (n, wc, ns, ns), its average over the chains)."""
        ns = self.setups[0].n_species
        wc = self._samp_wc
        per = np.zeros((self.n, wc, ns, ns), dtype=np.float64)
        av = np.zeros((wc, ns, ns), dtype=np.float64)
        _check(load().brawl_batch_asro_stats(self._h, int(n_save_asro), _ptr(per), _ptr(av)))
        return per, av

    # -- ALRO (store_state) of every chain --------------------------------------
    def alro_add(self) -> None:
        _check(load().brawl_batch_alro_add(self._h))

    def alro_reset(self) -> None:
        _check(load().brawl_batch_alro_reset(self._h))

    def alro(self, c: int) -> np.ndarray:
        s = self.setups[c]
        out = np.zeros(s.grid_shape + (1, s.n_species), dtype=np.float64)
        _check(load().brawl_batch_alro_get(self._h, c, _ptr(out)))
        return out


class NestedSampling:
    """Independent nested-sampling runs resident on the GPU (brawl_ns):
    nested_sampling_main (src/nested_sampling.f90:45-206)."""

    def __init__(self, runs: list[dict]):
        """Each run: dict(setup=Setup, V=array, seed=int, n_walkers=int,
        n_steps=int, species_concentrations=array, species_numbers=array|None)."""
        n = len(runs)
        descs = (_NsDesc * n)()
        keep = []
        self.runs = runs
        for k, r in enumerate(runs):
            s = r["setup"]
            V = _v_array(s, r["V"])
            conc = np.ascontiguousarray(r["species_concentrations"], dtype=np.float64)
            keep += [V, conc]
            d = descs[k]
            d.setup = s.c()
            d.V_ex = V.ctypes.data
            d.seed = int(r.get("seed", 5489)) & 0xFFFFFFFF
            d.n_walkers = int(r["n_walkers"])
            d.n_steps = int(r["n_steps"])
            d.species_concentrations = conc.ctypes.data
            nums = r.get("species_numbers")
            if nums is not None:
                nums = np.ascontiguousarray(nums, dtype=np.int64)
                keep.append(nums)
                d.species_numbers = nums.ctypes.data
        h = C.c_void_p()
        _check(load().brawl_ns_create(descs, n, C.byref(h)))
        self._h = h
        self.n = n

    def close(self):
        if getattr(self, "_h", None):
            load().brawl_ns_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def iterate(self, n_iter: int) -> np.ndarray:
        """Ceilings of the next n_iter iterations, shaped (runs, n_iter)."""
        out = np.zeros((self.n, n_iter), dtype=np.float64)
        _check(load().brawl_ns_iterate(self._h, int(n_iter), _ptr(out)))
        return out

    def energies(self, run: int) -> np.ndarray:
        out = np.zeros(int(self.runs[run]["n_walkers"]), dtype=np.float64)
        _check(load().brawl_ns_energies(self._h, run, _ptr(out)))
        return out

    def walker_config(self, run: int, walker: int) -> np.ndarray:
        out = np.zeros(self.runs[run]["setup"].grid_shape, dtype=np.int8)
        _check(load().brawl_ns_walker_config(self._h, run, walker, _ptr(out)))
        return out

    def counters(self, run: int) -> dict:
        c = np.zeros(NUM_COUNTERS, dtype=np.int64)
        _check(load().brawl_ns_counters(self._h, run, _ptr(c)))
        return dict(zip(COUNTER_NAMES, (int(v) for v in c)))


class WangLandauWalkers:
    """Wang-Landau walkers resident on the GPU (brawl_wl): sweeps() of
    every walker and the in-window averages (src/wang-landau.F90:539-632)."""

    def __init__(self, walkers: list[dict], bin_edges):
        """Each walker: dict(setup, V, seed, config, start_idx, end_idx,
        window, nbr_swap=False); bin_edges has bins+1 entries."""
        n = len(walkers)
        descs = (_WlDesc * n)()
        keep = []
        self.walkers = [dict(w) for w in walkers]  # windows may change (set_windows)
        for k, w in enumerate(walkers):
            s = w["setup"]
            V = _v_array(s, w["V"])
            cfg = np.ascontiguousarray(w["config"], dtype=np.int8)
            keep += [V, cfg]
            d = descs[k]
            d.setup = s.c()
            d.V_ex = V.ctypes.data
            d.seed = int(w["seed"]) & 0xFFFFFFFF
            d.config = cfg.ctypes.data
            d.start_idx = int(w["start_idx"])
            d.end_idx = int(w["end_idx"])
            d.window = int(w["window"])
            d.nbr_swap = int(bool(w.get("nbr_swap", False)))
        self.bin_edges = np.ascontiguousarray(bin_edges, dtype=np.float64)
        self.bins = self.bin_edges.size - 1
        h = C.c_void_p()
        _check(load().brawl_wl_create(descs, n, self.bins, _ptr(self.bin_edges), C.byref(h)))
        self._h = h
        self.n = n

    def close(self):
        if getattr(self, "_h", None):
            load().brawl_wl_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sweeps(self, n_trials: int, wl_f: float, hist_period: int) -> np.ndarray:
        acc = np.zeros(self.n, dtype=np.int64)
        _check(load().brawl_wl_sweeps(self._h, int(n_trials), float(wl_f), int(hist_period), _ptr(acc)))
        return acc

    def average(self) -> None:
        """dos_average: ln g averaged over each window's walkers."""
        _check(load().brawl_wl_average(self._h))

    def replica_exchange(self) -> tuple[int, np.ndarray, np.ndarray]:
        """replica_exchange: (accepted pairs, partner per walker or -1,
        exchanged flag per walker)."""
        partner = np.zeros(self.n, dtype=np.int32)
        exch = np.zeros(self.n, dtype=np.int32)
        na = C.c_int()
        _check(load().brawl_wl_replica_exchange(self._h, _ptr(partner), _ptr(exch), C.byref(na)))
        return int(na.value), partner, exch

    def flatness(self) -> np.ndarray:
        out = np.zeros(self.n, dtype=np.float64)
        _check(load().brawl_wl_flatness(self._h, _ptr(out)))
        return out

    def dos_combine(self) -> np.ndarray:
        """dos_combine: the stitched ln g, also written to every walker."""
        out = np.zeros(self.bins, dtype=np.float64)
        _check(load().brawl_wl_dos_combine(self._h, _ptr(out)))
        return out

    def reset_hist(self) -> None:
        _check(load().brawl_wl_reset_hist(self._h))

    def lng(self, w: int) -> np.ndarray:
        out = np.zeros(self.bins, dtype=np.float64)
        _check(load().brawl_wl_get_lng(self._h, w, _ptr(out)))
        return out

    def set_lng(self, w: int, lng) -> None:
        a = np.ascontiguousarray(lng, dtype=np.float64)
        _check(load().brawl_wl_set_lng(self._h, w, _ptr(a)))

    def hist(self, w: int) -> np.ndarray:
        nb = int(self.walkers[w]["end_idx"]) - int(self.walkers[w]["start_idx"]) + 1
        out = np.zeros(nb, dtype=np.float64)
        _check(load().brawl_wl_get_hist(self._h, w, _ptr(out)))
        return out

    def set_hist(self, w: int, hist) -> None:
        a = np.ascontiguousarray(hist, dtype=np.float64)
        _check(load().brawl_wl_set_hist(self._h, w, _ptr(a)))

    def energies(self) -> np.ndarray:
        out = np.zeros(self.n, dtype=np.float64)
        _check(load().brawl_wl_energies(self._h, _ptr(out)))
        return out

    def config(self, w: int) -> np.ndarray:
        out = np.zeros(self.walkers[w]["setup"].grid_shape, dtype=np.int8)
        _check(load().brawl_wl_get_config(self._h, w, _ptr(out)))
        return out

    def set_config(self, w: int, cfg) -> None:
        a = np.ascontiguousarray(cfg, dtype=np.int8)
        _check(load().brawl_wl_set_config(self._h, w, _ptr(a)))

    def swap_configs(self, a: int, b: int) -> None:
        _check(load().brawl_wl_swap_configs(self._h, a, b))

    def genrand(self, w: int, n: int) -> np.ndarray:
        out = np.zeros(n, dtype=np.float64)
        _check(load().brawl_wl_genrand(self._h, w, int(n), _ptr(out)))
        return out

    def counters(self, w: int) -> dict:
        c = np.zeros(NUM_COUNTERS, dtype=np.int64)
        _check(load().brawl_wl_counters(self._h, w, _ptr(c)))
        return dict(zip(COUNTER_NAMES, (int(v) for v in c)))

    # -- enter_energy_window (src/wang-landau.F90:643-741) -----------------------
    def enter_windows(self, energy_min: float, energy_max: float, species_concentrations,
                      species_numbers=None, initial: bool = True, max_steps: int = 10 ** 8) -> np.ndarray:
        """The biased walk of every walker into its window (energy range in
        meV/atom as wl_input gives it); returns the iterations each took."""
        conc = np.ascontiguousarray(species_concentrations, dtype=np.float64)
        nums = None if species_numbers is None else np.ascontiguousarray(species_numbers, dtype=np.int64)
        steps = np.zeros(self.n, dtype=np.int64)
        _check(load().brawl_wl_enter_windows(self._h, float(energy_min), float(energy_max), _ptr(conc),
                                             None if nums is None else _ptr(nums), int(bool(initial)),
                                             int(max_steps), _ptr(steps)))
        return steps

    # -- radial-density samples inside sweeps() (src/wang-landau.F90:566-586) --
    def radial_enable(self, wc_range: int, shells, radial_samples: int, num_walkers: int) -> None:
        sh = np.ascontiguousarray(shells, dtype=np.float64)
        if sh.size != wc_range:
            raise ValueError("shells needs wc_range entries")
        _check(load().brawl_wl_radial_enable(self._h, int(wc_range), _ptr(sh), int(radial_samples),
                                             int(num_walkers)))
        self.radial_wc = int(wc_range)

    def radial_set_done(self, done) -> None:
        """radial_record_bool (bins); every bin set stops the sampling."""
        d = np.ascontiguousarray(np.asarray(done, dtype=bool).astype(np.uint8))
        _check(load().brawl_wl_radial_set_done(self._h, _ptr(d)))

    def radial(self, w: int) -> tuple[np.ndarray, np.ndarray, int]:
        """(radial_record (bins), rho_of_E shaped (bins, wc, ns, ns) -- the C
        view of rho_of_E(i, j, l, bin) --, radial_mc_steps) of walker w."""
        ns = self.walkers[w]["setup"].n_species
        rec = np.zeros(self.bins, dtype=np.int32)
        rho = np.zeros((self.bins, self.radial_wc, ns, ns), dtype=np.float64)
        st = np.zeros(1, dtype=np.int32)
        _check(load().brawl_wl_radial_get(self._h, w, _ptr(rec), _ptr(rho), _ptr(st)))
        return rec, rho, int(st[0])

    # -- the configuration store (config_per_bin, src/wang-landau.F90:605-622) --
    def store_enable(self) -> None:
        """Every walker's per-bin configuration slots, all open."""
        _check(load().brawl_wl_store_enable(self._h))

    def store_flags(self) -> np.ndarray:
        """config_store of every walker: (n, bins) bool, True = open."""
        out = np.zeros((self.n, self.bins), dtype=np.uint8)
        _check(load().brawl_wl_store_flags(self._h, _ptr(out)))
        return out.astype(bool)

    def store_merge(self, pick) -> None:
        """merge_configs' copies: pick[bin - 1] is the walker whose slot
        every walker takes, or -1 (the bin reopens)."""
        p = np.ascontiguousarray(pick, dtype=np.int32)
        if p.size != self.bins:
            raise ValueError("pick needs one entry per bin")
        _check(load().brawl_wl_store_merge(self._h, _ptr(p)))

    def store_load(self, w: int, bin_1based: int) -> None:
        """load_window_config: walker w takes its stored configuration of the bin."""
        _check(load().brawl_wl_store_load(self._h, int(w), int(bin_1based)))

    def store_config(self, w: int, bin_1based: int) -> np.ndarray:
        """Walker w's stored configuration of the bin, (2n3, 2n2, 2n1) as config()."""
        out = np.zeros(self.walkers[w]["setup"].grid_shape, dtype=np.int8)
        _check(load().brawl_wl_store_get(self._h, int(w), int(bin_1based), _ptr(out)))
        return out

    def set_windows(self, start_idx, end_idx) -> None:
        """Per window, the new 1-based [start, end] (overlap included); the
        histograms restart from 0, ln g is kept."""
        a = np.ascontiguousarray(start_idx, dtype=np.int32)
        b = np.ascontiguousarray(end_idx, dtype=np.int32)
        _check(load().brawl_wl_set_windows(self._h, _ptr(a), _ptr(b)))
        win = [d["window"] for d in self.walkers]
        first = {}
        for k, wi in enumerate(win):
            first.setdefault(wi, len(first))
        for k, d in enumerate(self.walkers):
            j = first[d["window"]]
            d["start_idx"], d["end_idx"] = int(a[j]), int(b[j])
