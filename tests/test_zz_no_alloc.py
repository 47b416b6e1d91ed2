"""brawl_total_energy_noalloc: the total energy for callers that cannot let
a library allocate device memory (a host whose memory pool owns the whole
device, or one that records its GPU work into a CUDA graph).  The test owns
every device buffer; the entry point must agree exactly with
brawl_total_energy on two calls in a row (the second smaller than the
first, so stale scratch would show), and refuse a lattice larger than its
fixed scratch.  Kept in its own file so that it runs after every other test
when pytest collects alphabetically."""
import ctypes as C

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


def test_total_energy_noalloc_matches_existing_entry_point():
    import torch
    lib = B.load()
    cases = [("bcc", (10, 9, 8), 4, 6, 11), ("fcc", (3, 4, 2), 3, 4, 12)]
    for lattice, n, ns, nsh, seed in cases:          # two calls in a row
        V, cfg, mod = _system(lattice, n, ns, nsh, seed)
        setup = B.Setup(lattice, *n, ns, nsh)
        ch = B.Chain(setup, V)
        ch.set_config(cfg)
        expect = ch.total_energy()
        assert expect == mod.total_energy(cfg)
        dV = torch.from_numpy(np.ascontiguousarray(V.ravel(order="F"))).cuda()
        dcfg = torch.from_numpy(cfg.copy()).cuda()
        dE = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        s = setup.c()
        rc = lib.brawl_total_energy_noalloc(C.byref(s), C.c_void_p(dV.data_ptr()),
                                            C.c_void_p(dcfg.data_ptr()),
                                            C.c_void_p(dE.data_ptr()), None)
        assert rc == 0, lib.brawl_last_error()
        torch.cuda.synchronize()
        assert float(dE.item()) == expect


def test_total_energy_noalloc_rejects_oversized_lattice():
    lib = B.load()
    s = B.Setup("fcc", 64, 64, 64, 2, 1).c()   # 1048576 sites > 524288
    rc = lib.brawl_total_energy_noalloc(C.byref(s), C.c_void_p(8), C.c_void_p(8),
                                        C.c_void_p(8), None)
    assert rc == 1
    assert b"exceed" in lib.brawl_last_error()
