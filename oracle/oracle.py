"""ctypes binding of the CPU oracle (oracle/brawl_oracle.c).

TEST INFRASTRUCTURE ONLY.  The oracle is the checker for the CUDA path: only
tests/, the smoke check in __graft_entry__ and the CPU-baseline leg of
bench.py import this module.  The brawl_gb300 package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_MT_PATH = os.path.join(HERE, "_ref", "libmt19937ar_ref.so")

SC, BCC, FCC = 0, 1, 2
LATTICE_IDS = {"simple_cubic": SC, "sc": SC, "bcc": BCC, "fcc": FCC}


def reference_dir() -> str:
    """Where a checkout of the reference is looked for: $BRAWL_REFERENCE_DIR,
    else a `reference` directory beside this repository."""
    env = os.environ.get("BRAWL_REFERENCE_DIR")
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and, with ref=True, the reference's own
    mt19937ar.c into _ref/ where its sources are present) with the committed
    Makefile."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref-if-present", "REF_DIR=" + reference_dir()],
                       check=True)


class Rng(C.Structure):
    _fields_ = [("mt", C.c_uint32 * 624), ("mti", C.c_int)]


class Model(C.Structure):
    _fields_ = [("lattice", C.c_int), ("n1", C.c_int), ("n2", C.c_int), ("n3", C.c_int),
                ("nsh", C.c_int), ("ns", C.c_int), ("V", C.POINTER(C.c_double))]


class Counters(C.Structure):
    _fields_ = [("trials", C.c_int64), ("evaluated", C.c_int64), ("draws", C.c_int64),
                ("accepted", C.c_int64), ("exp_tests", C.c_int64)]


class AnnealParams(C.Structure):
    _fields_ = [("T", C.c_double), ("delta_T", C.c_double), ("T_steps", C.c_int),
                ("n_mc_steps", C.c_int64), ("n_burn_in_steps", C.c_int64),
                ("n_sample_steps", C.c_int64), ("n_sample_steps_asro", C.c_int64),
                ("n_sample_steps_alro", C.c_int64), ("n_sample_steps_trajectory", C.c_int64),
                ("burn_in", C.c_int), ("burn_in_start", C.c_int),
                ("calculate_energies", C.c_int), ("calculate_asro", C.c_int),
                ("nbr_swap", C.c_int), ("wc_range", C.c_int)]


class AnnealOut(C.Structure):
    _fields_ = [("temperature", C.c_void_p), ("energies_of_T", C.c_void_p),
                ("C_of_T", C.c_void_p), ("acceptance_of_T", C.c_void_p),
                ("rho_of_T", C.c_void_p), ("traj_capacity", C.c_int64),
                ("traj_rows", C.c_int64), ("traj_step", C.c_void_p),
                ("traj_energy", C.c_void_p), ("traj_asro", C.c_void_p),
                ("initial_configs", C.c_void_p), ("final_configs", C.c_void_p),
                ("shells", C.c_void_p)]


class NsParams(C.Structure):
    _fields_ = [("n_walkers", C.c_int), ("n_steps", C.c_int), ("n_iter", C.c_int)]


class WlRadial(C.Structure):
    _fields_ = [("wc_range", C.c_int), ("shells", C.c_void_p), ("cap", C.c_int), ("done", C.c_void_p),
                ("record", C.c_void_p), ("rho_of_E", C.c_void_p), ("steps", C.c_void_p)]


class WlStore(C.Structure):
    _fields_ = [("slots", C.c_void_p), ("open", C.c_void_p), ("cfg_bytes", C.c_size_t)]


class WlParams(C.Structure):
    _fields_ = [("bins", C.c_int), ("start_idx", C.c_int), ("end_idx", C.c_int),
                ("n_trials", C.c_int64), ("wl_f", C.c_double), ("hist_period", C.c_int),
                ("nbr_swap", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        vp, i64, dp = C.c_void_p, C.c_int64, C.c_double
        L.bo_rng_seed.argtypes = [C.POINTER(Rng), C.c_uint32]
        L.bo_rng_u32.argtypes = [C.POINTER(Rng)]
        L.bo_rng_u32.restype = C.c_uint32
        L.bo_rng_uniform.argtypes = [C.POINTER(Rng)]
        L.bo_rng_uniform.restype = dp
        L.bo_static_seed.restype = C.c_uint32
        L.bo_n_atoms.argtypes = [C.POINTER(Model)]
        L.bo_grid_size.argtypes = [C.POINTER(Model)]
        L.bo_shell_size.argtypes = [C.c_int, C.c_int]
        L.bo_shell_offset.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]
        L.bo_site_energy.argtypes = [C.POINTER(Model), vp, C.c_int, C.c_int, C.c_int]
        L.bo_site_energy.restype = dp
        L.bo_pair_energy.argtypes = [C.POINTER(Model), vp, vp, vp]
        L.bo_pair_energy.restype = dp
        L.bo_total_energy.argtypes = [C.POINTER(Model), vp]
        L.bo_total_energy.restype = dp
        L.bo_random_site.argtypes = [C.POINTER(Model), C.POINTER(Rng), vp]
        L.bo_mc_step.argtypes = [C.POINTER(Model), vp, C.POINTER(Rng), dp, C.c_int,
                                 C.POINTER(Counters)]
        L.bo_mc_run.argtypes = [C.POINTER(Model), vp, C.POINTER(Rng), dp, i64, C.c_int,
                                C.POINTER(Counters)]
        L.bo_mc_run.restype = i64
        L.bo_mc_trace.argtypes = [C.POINTER(Model), vp, C.POINTER(Rng), dp, i64, C.c_int, vp, vp,
                                  C.POINTER(Counters)]
        L.bo_mc_trace.restype = i64
        L.bo_initial_setup.argtypes = [C.POINTER(Model), vp, vp, C.POINTER(Rng), vp]
        L.bo_lattice_shells.argtypes = [C.POINTER(Model), vp, C.c_int, vp]
        L.bo_radial_densities.argtypes = [C.POINTER(Model), vp, C.c_int, vp, vp, vp]
        L.bo_anneal.argtypes = [C.POINTER(Model), C.POINTER(AnnealParams), vp, C.POINTER(Rng),
                                C.POINTER(AnnealOut)]
        L.bo_ns_run.argtypes = [C.POINTER(Model), C.POINTER(NsParams), vp, vp, C.POINTER(Rng), vp,
                                vp, vp, vp]
        L.bo_ns_walk.argtypes = [C.POINTER(Model), vp, C.POINTER(Rng), vp, dp, i64,
                                 C.POINTER(Counters)]
        L.bo_ns_walk.restype = i64
        L.bo_wl_bin_index.argtypes = [dp, vp, C.c_int]
        L.bo_wl_sweep.argtypes = [C.POINTER(Model), C.POINTER(WlParams), vp, C.POINTER(Rng), vp,
                                  vp, vp, vp, C.POINTER(Counters)]
        L.bo_wl_sweep.restype = i64
        L.bo_wl_sweep_radial.argtypes = [C.POINTER(Model), C.POINTER(WlParams), vp, C.POINTER(Rng), vp,
                                         vp, vp, vp, C.POINTER(Counters), C.POINTER(WlRadial)]
        L.bo_wl_sweep_radial.restype = i64
        L.bo_wl_sweep_store.argtypes = [C.POINTER(Model), C.POINTER(WlParams), vp, C.POINTER(Rng), vp,
                                        vp, vp, vp, C.POINTER(Counters), C.POINTER(WlRadial),
                                        C.POINTER(WlStore)]
        L.bo_wl_sweep_store.restype = i64
        L.bo_wl_enter_window.argtypes = [C.POINTER(Model), vp, C.POINTER(Rng), vp, vp, dp, dp, dp, i64, vp]
        L.bo_wl_enter_window.restype = i64
        L.bo_wl_replica_exchange.argtypes = [C.c_int, C.c_int, vp, vp, vp, C.c_int, vp, vp,
                                             C.POINTER(Rng), vp, C.c_size_t, vp, vp]
        L.bo_wl_dos_combine.argtypes = [C.c_int, vp, vp, C.c_int, vp, vp]
        L.bo_wl_flatness.argtypes = [vp, C.c_int]
        L.bo_wl_flatness.restype = dp
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class OracleRng:
    """One mt19937ar stream (a copy of the reference's global generator)."""

    def __init__(self, seed: int):
        self.s = Rng()
        lib().bo_rng_seed(C.byref(self.s), seed)

    def u32(self) -> int:
        return lib().bo_rng_u32(C.byref(self.s))

    def uniform(self) -> float:
        return lib().bo_rng_uniform(C.byref(self.s))

    def state_words(self) -> np.ndarray:
        """624 words + index, the layout the C-ABI's rng get/set uses."""
        out = np.zeros(625, dtype=np.uint32)
        out[:624] = np.frombuffer(bytes(self.s.mt), dtype=np.uint32)
        out[624] = self.s.mti
        return out

    def set_state_words(self, words: np.ndarray) -> None:
        w = np.ascontiguousarray(words, dtype=np.uint32)
        for i in range(624):
            self.s.mt[i] = int(w[i])
        self.s.mti = int(w[624])


class OracleModel:
    """Lattice + interactions in the reference's layout."""

    def __init__(self, lattice, n1, n2, n3, V: np.ndarray):
        lat = LATTICE_IDS[lattice] if isinstance(lattice, str) else int(lattice)
        V = np.asfortranarray(np.asarray(V, dtype=np.float64))
        assert V.ndim == 3 and V.shape[0] == V.shape[1]
        self.V = np.ascontiguousarray(V.ravel(order="F"))
        self.ns = V.shape[0]
        self.nsh = V.shape[2]
        self.lattice = lat
        self.n = (n1, n2, n3)
        self.m = Model(lat, n1, n2, n3, self.nsh, self.ns, self.V.ctypes.data_as(C.POINTER(C.c_double)))

    @property
    def grid_shape(self):
        """(z, y, x) shape of a C-ordered view of config(1, x, y, z)."""
        n1, n2, n3 = self.n
        return (2 * n3, 2 * n2, 2 * n1)

    @property
    def n_atoms(self) -> int:
        return lib().bo_n_atoms(C.byref(self.m))

    def empty_config(self) -> np.ndarray:
        return np.zeros(self.grid_shape, dtype=np.int8)

    def total_energy(self, cfg: np.ndarray) -> float:
        assert cfg.dtype == np.int8 and cfg.flags.c_contiguous
        return lib().bo_total_energy(C.byref(self.m), _ptr(cfg))

    def site_energy(self, cfg, x, y, z) -> float:
        return lib().bo_site_energy(C.byref(self.m), _ptr(cfg), x, y, z)

    def pair_energy(self, cfg, a, b) -> float:
        a = np.asarray(a, dtype=np.int32)
        b = np.asarray(b, dtype=np.int32)
        return lib().bo_pair_energy(C.byref(self.m), _ptr(cfg), _ptr(a), _ptr(b))

    def random_site(self, rng: OracleRng):
        s = np.zeros(3, dtype=np.int32)
        lib().bo_random_site(C.byref(self.m), C.byref(rng.s), _ptr(s))
        return tuple(int(v) for v in s)

    def initial_setup(self, rng: OracleRng, conc, numbers=None) -> tuple[np.ndarray, np.ndarray]:
        conc = np.ascontiguousarray(np.asarray(conc, dtype=np.float64)).copy()
        assert conc.shape == (self.ns + 1,)
        nums = None if numbers is None else np.ascontiguousarray(np.asarray(numbers, dtype=np.int64))
        cfg = self.empty_config()
        rc = lib().bo_initial_setup(C.byref(self.m), _ptr(conc), None if nums is None else _ptr(nums),
                                    C.byref(rng.s), _ptr(cfg))
        if rc != 0:
            raise ValueError("initial_setup: species counts do not sum to the number of sites")
        return cfg, conc

    def mc_run(self, cfg, rng, beta, n_trials, nbr_swap=False) -> tuple[int, Counters]:
        c = Counters()
        acc = lib().bo_mc_run(C.byref(self.m), _ptr(cfg), C.byref(rng.s), beta, n_trials,
                              int(nbr_swap), C.byref(c))
        return acc, c

    def mc_trace(self, cfg, rng, beta, n_trials, nbr_swap=False):
        acc = np.zeros(n_trials, dtype=np.int8)
        de = np.zeros(n_trials, dtype=np.float64)
        c = Counters()
        lib().bo_mc_trace(C.byref(self.m), _ptr(cfg), C.byref(rng.s), beta, n_trials, int(nbr_swap),
                          _ptr(acc), _ptr(de), C.byref(c))
        return acc, de, c

    def lattice_shells(self, cfg, wc_range) -> np.ndarray:
        out = np.zeros(wc_range, dtype=np.float64)
        lib().bo_lattice_shells(C.byref(self.m), _ptr(cfg), wc_range, _ptr(out))
        return out

    def radial_densities(self, cfg, shells) -> tuple[np.ndarray, np.ndarray]:
        """rho and raw counts, both shaped (wc, ns, ns) = C view of rho(i, j, l)."""
        shells = np.ascontiguousarray(shells, dtype=np.float64)
        wc = shells.shape[0]
        rho = np.zeros((wc, self.ns, self.ns), dtype=np.float64)
        cnt = np.zeros((wc, self.ns, self.ns), dtype=np.int64)
        lib().bo_radial_densities(C.byref(self.m), _ptr(cfg), wc, _ptr(shells), _ptr(rho), _ptr(cnt))
        return rho, cnt

    def anneal(self, cfg, rng, params: dict, traj_capacity=None):
        p = AnnealParams(**params)
        Ts = p.T_steps
        ns, wc = self.ns, p.wc_range
        if traj_capacity is None:
            traj_capacity = Ts * (p.n_mc_steps // p.n_sample_steps_trajectory + 1)
        out = {
            "temperature": np.zeros(Ts), "energies_of_T": np.zeros(Ts), "C_of_T": np.zeros(Ts),
            "acceptance_of_T": np.zeros(Ts), "rho_of_T": np.zeros((Ts, wc, ns, ns)),
            "traj_step": np.zeros(traj_capacity, dtype=np.int64),
            "traj_energy": np.zeros(traj_capacity),
            "traj_asro": np.zeros((traj_capacity, wc, ns, ns)),
            "initial_configs": np.zeros((Ts,) + self.grid_shape, dtype=np.int8),
            "final_configs": np.zeros((Ts,) + self.grid_shape, dtype=np.int8),
            "shells": np.zeros(wc),
        }
        o = AnnealOut()
        for k, v in out.items():
            setattr(o, k, v.ctypes.data)
        o.traj_capacity = traj_capacity
        rc = lib().bo_anneal(C.byref(self.m), C.byref(p), _ptr(cfg), C.byref(rng.s), C.byref(o))
        assert rc == 0
        rows = o.traj_rows
        for k in ("traj_step", "traj_energy", "traj_asro"):
            out[k] = out[k][:rows]
        return out

    def ns_run(self, rng, conc, numbers, n_walkers, n_steps, n_iter):
        conc = np.ascontiguousarray(np.asarray(conc, dtype=np.float64)).copy()
        nums = None if numbers is None else np.ascontiguousarray(np.asarray(numbers, dtype=np.int64))
        walkers = np.zeros((n_walkers,) + self.grid_shape, dtype=np.int8)
        energies = np.zeros(n_walkers)
        limits = np.zeros(n_iter)
        acc = np.zeros(1, dtype=np.int64)
        p = NsParams(n_walkers, n_steps, n_iter)
        rc = lib().bo_ns_run(C.byref(self.m), C.byref(p), _ptr(conc), None if nums is None else _ptr(nums),
                             C.byref(rng.s), _ptr(walkers), _ptr(energies), _ptr(limits), _ptr(acc))
        assert rc == 0
        return limits, walkers, energies, int(acc[0])

    def ns_walk(self, cfg, rng, energy, ener_limit, n_steps):
        e = np.array([energy], dtype=np.float64)
        c = Counters()
        acc = lib().bo_ns_walk(C.byref(self.m), _ptr(cfg), C.byref(rng.s), _ptr(e), ener_limit, n_steps,
                               C.byref(c))
        return acc, float(e[0]), c

    def wl_enter_window(self, cfg, rng, conc, numbers, min_e, max_e, sig2x2, max_steps):
        """enter_energy_window for one walker: (iterations or -1, energy)."""
        conc = np.ascontiguousarray(np.asarray(conc, dtype=np.float64))
        nums = None if numbers is None else np.ascontiguousarray(np.asarray(numbers, dtype=np.int64))
        e = np.zeros(1)
        it = lib().bo_wl_enter_window(C.byref(self.m), _ptr(cfg), C.byref(rng.s), _ptr(conc),
                                      None if nums is None else _ptr(nums), float(min_e), float(max_e),
                                      float(sig2x2), int(max_steps), _ptr(e))
        return int(it), float(e[0])

    def wl_sweep(self, cfg, rng, bin_edges, lng, hist, energy, bins, start_idx, end_idx, n_trials,
                 wl_f, hist_period, nbr_swap=False, radial=None, store=None):
        """radial (optional): dict(shells, cap, done (uint8, bins), record
        (int32, bins), rho_of_E (float64, (bins, wc, ns, ns)), steps (int32,
        1)), updated in place.  store (optional): dict(slots (int8, (bins,)
        + cfg.shape), open (uint8, bins)), config_per_bin and config_store,
        updated in place."""
        e = np.array([energy], dtype=np.float64)
        p = WlParams(bins, start_idx, end_idx, n_trials, wl_f, hist_period, int(bool(nbr_swap)))
        c = Counters()
        rad = None
        if radial is not None:
            for k, dt in (("shells", np.float64), ("done", np.uint8), ("record", np.int32),
                          ("rho_of_E", np.float64), ("steps", np.int32)):
                a = radial[k]
                assert a.dtype == dt and a.flags.c_contiguous, k
            rad = WlRadial(radial["shells"].size, radial["shells"].ctypes.data, int(radial["cap"]),
                           radial["done"].ctypes.data, radial["record"].ctypes.data,
                           radial["rho_of_E"].ctypes.data, radial["steps"].ctypes.data)
        st = None
        if store is not None:
            sl, op = store["slots"], store["open"]
            assert sl.dtype == np.int8 and sl.flags.c_contiguous and sl.shape[0] == bins
            assert op.dtype == np.uint8 and op.flags.c_contiguous and op.size == bins
            st = WlStore(sl.ctypes.data, op.ctypes.data, cfg.size)
        acc = lib().bo_wl_sweep_store(C.byref(self.m), C.byref(p), _ptr(cfg), C.byref(rng.s),
                                      _ptr(bin_edges), _ptr(lng), _ptr(hist), _ptr(e), C.byref(c),
                                      None if rad is None else C.byref(rad),
                                      None if st is None else C.byref(st))
        return acc, float(e[0]), c


def wl_bin_index(energy, bin_edges, bins) -> int:
    be = np.ascontiguousarray(bin_edges, dtype=np.float64)
    return lib().bo_wl_bin_index(energy, _ptr(be), bins)


def wl_replica_exchange(win_start, win_end, per_window, bin_edges, energies, lngs, rngs, cfgs):
    """replica_exchange over walkers ordered by window.  lngs: list of ln g
    arrays (read only); rngs: list of OracleRng (advanced in place); cfgs:
    list of equal-shape configurations (swapped in place).  Returns
    (n_accepted, partner, accepted)."""
    n_windows = len(win_start)
    n = n_windows * per_window
    assert len(lngs) == n and len(rngs) == n and len(cfgs) == n
    ws = np.ascontiguousarray(win_start, dtype=np.int32)
    we = np.ascontiguousarray(win_end, dtype=np.int32)
    be = np.ascontiguousarray(bin_edges, dtype=np.float64)
    e = np.ascontiguousarray(energies, dtype=np.float64)
    L = np.ascontiguousarray(np.stack(lngs), dtype=np.float64)
    arr = (Rng * n)()
    for k, r in enumerate(rngs):
        C.memmove(C.byref(arr[k]), C.byref(r.s), C.sizeof(Rng))
    cf = np.ascontiguousarray(np.stack(cfgs))
    partner = np.zeros(n, dtype=np.int32)
    acc = np.zeros(n, dtype=np.int32)
    na = lib().bo_wl_replica_exchange(n_windows, per_window, _ptr(ws), _ptr(we), _ptr(be), be.size - 1,
                                      _ptr(e), _ptr(L), arr, _ptr(cf), cf[0].nbytes, _ptr(partner),
                                      _ptr(acc))
    for k, r in enumerate(rngs):
        C.memmove(C.byref(r.s), C.byref(arr[k]), C.sizeof(Rng))
    for k in range(n):
        cfgs[k][...] = cf[k]
    return na, partner, acc


def wl_dos_combine(win_start, win_end, lng_windows):
    """dos_combine: lng_windows is one ln g per window (n_windows x bins)."""
    ws = np.ascontiguousarray(win_start, dtype=np.int32)
    we = np.ascontiguousarray(win_end, dtype=np.int32)
    L = np.ascontiguousarray(lng_windows, dtype=np.float64)
    out = np.zeros(L.shape[1], dtype=np.float64)
    rc = lib().bo_wl_dos_combine(len(ws), _ptr(ws), _ptr(we), L.shape[1], _ptr(L), _ptr(out))
    if rc != 0:
        raise ValueError("a window has no overlap with the previous one")
    return out


def wl_flatness(hist) -> float:
    h = np.ascontiguousarray(hist, dtype=np.float64)
    return lib().bo_wl_flatness(_ptr(h), h.size)


def shell_offsets(lattice, shell):
    lat = LATTICE_IDS[lattice] if isinstance(lattice, str) else int(lattice)
    n = lib().bo_shell_size(lat, shell)
    out = []
    d = (C.c_int * 3)()
    for k in range(n):
        lib().bo_shell_offset(lat, shell, k, d)
        out.append((d[0], d[1], d[2]))
    return out


def reference_mt_words(seed: int, n: int) -> np.ndarray:
    """n words from the reference's own src/mt19937ar.c (compiled into _ref/),
    seeded with its init_genrand."""
    L = C.CDLL(REF_MT_PATH)
    L.init_genrand.argtypes = [C.c_ulong]
    L.genrand_int32.restype = C.c_ulong
    L.init_genrand(seed)
    return np.array([L.genrand_int32() & 0xFFFFFFFF for _ in range(n)], dtype=np.uint32)
