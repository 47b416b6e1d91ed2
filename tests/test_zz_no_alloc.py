"""brawl_total_energy_noalloc: the total energy for callers that cannot let
a library allocate device memory (a host whose memory pool owns the whole
device, or one that records its GPU work into a CUDA graph).  The test owns
every device buffer; the entry point must agree exactly with
brawl_total_energy and with the oracle on calls in a row (each smaller than
the one before, so stale scratch would show), on every lattice (simple cubic
included, whose neighbour wrap differs from its grid stride), on the default
stream, on a stream of the caller's and from a thread that has not used CUDA
before, and refuse a lattice larger than its fixed scratch.  Kept in its own
file so that it runs after every other test when pytest collects
alphabetically."""
import ctypes as C
import threading

import numpy as np
import pytest

import brawl_gb300 as B
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _system(lattice, n, ns, nsh, seed):
    rng = np.random.default_rng(seed)
    V = np.zeros((ns, ns, nsh))
    for sh in range(nsh):
        a = rng.uniform(-0.05, 0.05, size=(ns, ns))
        V[:, :, sh] = (np.triu(a) + np.triu(a, 1).T) / B.RY_TO_EV
    mod = O.OracleModel(lattice, *n, V)
    r = O.OracleRng(seed)
    conc = np.array([0.0] + [1.0 / ns] * ns)
    cfg, _ = mod.initial_setup(r, conc)
    return V, cfg, mod


def _noalloc(lib, setup, V, cfg, stream=None):
    import torch
    dV = torch.from_numpy(np.ascontiguousarray(V.ravel(order="F"))).cuda()
    dcfg = torch.from_numpy(cfg.copy()).cuda()
    dE = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    s = setup.c()
    handle = None if stream is None else C.c_void_p(stream.cuda_stream)
    rc = lib.brawl_total_energy_noalloc(C.byref(s), C.c_void_p(dV.data_ptr()),
                                        C.c_void_p(dcfg.data_ptr()), C.c_void_p(dE.data_ptr()),
                                        handle)
    assert rc == 0, lib.brawl_last_error()
    if stream is None:
        torch.cuda.synchronize()
    else:
        stream.synchronize()
    return float(dE.item())


CASES = [("bcc", (10, 9, 8), 4, 6, 11), ("fcc", (3, 4, 2), 3, 4, 12),
         ("simple_cubic", (3, 4, 5), 3, 2, 13), ("bcc", (2, 3, 2), 2, 3, 14)]


def test_total_energy_noalloc_matches_existing_entry_point():
    import torch
    lib = B.load()
    for k, (lattice, n, ns, nsh, seed) in enumerate(CASES):   # calls in a row
        V, cfg, mod = _system(lattice, n, ns, nsh, seed)
        setup = B.Setup(lattice, *n, ns, nsh)
        ch = B.Chain(setup, V)
        ch.set_config(cfg)
        expect = ch.total_energy()
        assert expect == mod.total_energy(cfg)
        stream = torch.cuda.Stream() if k % 2 else None
        assert _noalloc(lib, setup, V, cfg, stream) == expect


def test_total_energy_noalloc_from_a_new_thread():
    lib = B.load()
    lattice, n, ns, nsh, seed = CASES[0]
    V, cfg, mod = _system(lattice, n, ns, nsh, seed)
    setup = B.Setup(lattice, *n, ns, nsh)
    out = {}

    def run():
        try:
            out["e"] = _noalloc(lib, setup, V, cfg)
        except BaseException as exc:   # reported in the main thread
            out["err"] = exc

    t = threading.Thread(target=run)
    t.start()
    t.join()
    assert "err" not in out, out.get("err")
    assert out["e"] == mod.total_energy(cfg)


def test_total_energy_noalloc_rejects_oversized_lattice():
    lib = B.load()
    s = B.Setup("fcc", 64, 64, 64, 2, 1).c()   # 1048576 sites > 524288
    rc = lib.brawl_total_energy_noalloc(C.byref(s), C.c_void_p(8), C.c_void_p(8),
                                        C.c_void_p(8), None)
    assert rc == 1
    assert b"exceed" in lib.brawl_last_error()
