"""The serving loop (brawl_serve_*): every job's results are the same run
alone and run in a mix with other jobs (bit for bit), they equal the
oracle's run of the same job, and jobs submitted while others are on the
GPU are admitted and run beside them."""
import time

import numpy as np
import pytest

import brawl_gb300 as B
from brawl_gb300 import serving as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _job(kind, lattice, L, ns, nsh, seed, **kw):
    rng = np.random.default_rng(seed)
    N = S.n_sites(lattice, L)
    counts = np.full(ns, N // ns, dtype=np.int64)
    counts[: N - counts.sum()] += 1
    job = {"kind": kind, "setup": B.Setup(lattice, L, L, L, ns, nsh),
           "V": S.symmetric_V(rng, ns, nsh, 0.05), "seed": seed,
           "conc": np.concatenate([[0.0], counts / N]), "numbers": counts,
           "lattice": lattice, "L": L, "N": N}
    job.update(kw)
    return job


def _jobs():
    return [
        _job("anneal", "bcc", 3, 3, 3, 11, T_start=1500.0, delta_T=-400.0, T_steps=3, sweeps_per_T=40),
        _job("anneal", "fcc", 3, 2, 2, 12, T_start=900.0, delta_T=-200.0, T_steps=4, sweeps_per_T=25),
        _job("anneal", "bcc", 5, 4, 6, 13, T_start=2000.0, delta_T=-500.0, T_steps=2, sweeps_per_T=30),
        _job("wl", "bcc", 3, 2, 2, 21, wl_walkers=2, wl_bins=32, wl_calls=6, wl_trials=1300,
             wl_half_width=0.3, wl_f=1.0, wl_flatness=0.3, wl_tolerance=1e-6),
        _job("wl", "fcc", 3, 3, 3, 22, wl_walkers=3, wl_bins=40, wl_calls=5, wl_trials=216,
             wl_half_width=0.5, wl_f=0.5, wl_flatness=0.2, wl_tolerance=1e-6),
        _job("ns", "fcc", 2, 3, 2, 31, ns_walkers=16, ns_steps=20, ns_iter=30),
        _job("ns", "bcc", 3, 2, 3, 32, ns_walkers=24, ns_steps=30, ns_iter=17),
    ]


def _collect(server, jid):
    r = server.wait(jid, timeout=300)
    assert r["status"] == 0, r
    out = dict(r)
    out["values"] = server.values(jid, r["n_values"])
    out["config"] = server.config(jid)
    server.release(jid)
    return out


def _same(a, b):
    for k in ("status", "kind", "trials", "accepted", "wl_halvings", "n_values"):
        assert a[k] == b[k], k
    for k in ("energy", "wl_f"):
        assert a[k] == b[k] or (np.isnan(a[k]) and np.isnan(b[k])), k
    assert np.array_equal(a["values"], b["values"])
    assert np.array_equal(a["config"], b["config"])


def _oracle(job):
    """The job run by the oracle the way the serving loop defines it."""
    lat, L = job["lattice"], job["L"]
    mod = O.OracleModel(lat, L, L, L, job["V"])
    N = job["N"]
    if job["kind"] == "anneal":
        rng = O.OracleRng(job["seed"])
        cfg, _ = mod.initial_setup(rng, job["conc"], job["numbers"])
        E, acc = [], []
        trials = job["sweeps_per_T"] * N
        for k in range(job["T_steps"]):
            T = job["T_start"] + k * job["delta_T"]
            a, _ = mod.mc_run(cfg, rng, 1.0 / (T * B.K_B_IN_RY), trials)
            E.append(mod.total_energy(cfg))
            acc.append(a / trials if trials else 0.0)
        return np.array(E + acc), cfg
    if job["kind"] == "wl":
        nw, bins = job["wl_walkers"], job["wl_bins"]
        rngs = [O.OracleRng(job["seed"] + 11 * k) for k in range(nw)]
        cfgs = [mod.initial_setup(r, job["conc"], job["numbers"])[0] for r in rngs]
        es = [mod.total_energy(c) for c in cfgs]
        c = 0.0
        for e in es:
            c = c + e
        c = c / nw
        hw = job["wl_half_width"]
        for e in es:
            hw = max(hw, 1.25 * abs(e - c))
        edges = np.array([(c - hw) + i * ((2.0 * hw) / bins) for i in range(bins + 1)])
        lngs = [np.zeros(bins) for _ in range(nw)]
        hists = [np.zeros(bins) for _ in range(nw)]
        f = job["wl_f"]
        period = int(0.02 * float(np.float32(N)))
        for call in range(job["wl_calls"]):
            for k in range(nw):
                mod.wl_sweep(cfgs[k], rngs[k], edges, lngs[k], hists[k], mod.total_energy(cfgs[k]), bins,
                             1, bins, job["wl_trials"], f, period)
            if nw > 1:
                inv = float(np.float32(nw))
                for arrs in (lngs, hists):
                    s = arrs[0].copy()
                    for k in range(1, nw):
                        s = s + arrs[k]
                    s = s / inv
                    for k in range(nw):
                        arrs[k][:] = s
            if all(O.wl_flatness(h) > job["wl_flatness"] for h in hists):
                f *= 0.5
                for h in hists:
                    h[:] = 0.0
            if f < job["wl_tolerance"]:
                break
        return np.concatenate([lngs[0], edges]), cfgs[0]
    rng = O.OracleRng(job["seed"])
    limits, walkers, _, _ = mod.ns_run(rng, job["conc"], job["numbers"], job["ns_walkers"], job["ns_steps"],
                                       job["ns_iter"])
    return limits, walkers[0]


def test_serving_results_alone_equal_results_in_the_mix_and_the_oracle():
    jobs = _jobs()
    with S.Server(max_trials=500, max_iterations=3) as srv:
        ids = [srv.submit(j) for j in jobs]
        mixed = [_collect(srv, i) for i in ids]
        assert srv.stats()["rounds"] > 5
    for job, m in zip(jobs, mixed):
        with S.Server() as srv:
            alone = _collect(srv, srv.submit(job))
        _same(alone, m)
        vals, cfg = _oracle(job)
        assert np.array_equal(m["values"], vals), job["kind"]
        assert np.array_equal(m["config"], cfg), job["kind"]
    # the mixed run really interleaved: every job was resident before the first ended
    first_end = min(m["t_finish"] for m in mixed)
    assert all(m["t_admit"] <= first_end for m in mixed)


def test_serving_admits_jobs_that_arrive_while_others_run():
    jobs = _jobs()
    long_job = _job("anneal", "fcc", 6, 3, 4, 41, T_start=1200.0, delta_T=-100.0, T_steps=3,
                    sweeps_per_T=300)
    with S.Server(max_trials=2000) as srv:
        lid = srv.submit(long_job)
        t0 = time.time()
        while srv.stats()["rounds"] < 2 and time.time() - t0 < 60:
            time.sleep(0.002)
        later = []
        for j in jobs:
            later.append(srv.submit(j))
            time.sleep(0.003)
        res_later = [_collect(srv, i) for i in later]
        res_long = _collect(srv, lid)
    assert res_long["t_finish"] > max(r["t_admit"] for r in res_later)
    for job, r in zip(jobs, res_later):
        vals, cfg = _oracle(job)
        assert np.array_equal(r["values"], vals)
        assert np.array_equal(r["config"], cfg)
    vals, cfg = _oracle(long_job)
    assert np.array_equal(res_long["values"], vals)


def test_serving_budget_queues_jobs_and_reports_bad_jobs():
    jobs = _jobs()[:3]
    # a budget below one job: jobs run one at a time, in arrival order
    with S.Server(hbm_budget=1) as srv:
        ids = [srv.submit(j) for j in jobs]
        res = [_collect(srv, i) for i in ids]
    for a, b in zip(res, res[1:]):
        assert b["t_admit"] >= a["t_finish"]
    for job, r in zip(jobs, res):
        vals, _ = _oracle(job)
        assert np.array_equal(r["values"], vals)
    bad = _job("anneal", "bcc", 3, 2, 2, 5, T_start=-10.0, delta_T=0.0, T_steps=1, sweeps_per_T=1)
    with S.Server() as srv:
        with pytest.raises(B.BrawlError) as ex:
            srv.submit(bad)
        assert ex.value.code == 1
        # a WL window narrower than the walkers' spread is widened to hold them all
        narrow = _job("wl", "bcc", 3, 2, 2, 9, wl_walkers=2, wl_bins=8, wl_calls=2, wl_trials=10,
                      wl_half_width=1e-12, wl_f=1.0, wl_flatness=0.5, wl_tolerance=1e-6)
        jid = srv.submit(narrow)
        r = srv.wait(jid, timeout=120)
        assert r["status"] == 0
        vals, _ = _oracle(narrow)
        assert np.array_equal(srv.values(jid, r["n_values"]), vals)


def test_serving_kind_caps_admit_past_a_capped_kind():
    """With one resident nested-sampling job allowed, the second and third
    wait for the first to end while the anneal jobs queued behind them are
    admitted at once; every job still equals the oracle's run."""
    jobs = _jobs()
    ns = [j for j in jobs if j["kind"] == "ns"]
    ns.append(_job("ns", "fcc", 2, 2, 2, 33, ns_walkers=12, ns_steps=16, ns_iter=12))
    anneals = [j for j in jobs if j["kind"] == "anneal"]
    order = ns + anneals
    with S.Server(max_active_ns=1, max_iterations=2) as srv:
        ids = [srv.submit(j) for j in order]
        res = [_collect(srv, i) for i in ids]
    r_ns, r_an = res[:len(ns)], res[len(ns):]
    # at most one nested-sampling job resident at a time, in arrival order
    for a, b in zip(r_ns, r_ns[1:]):
        assert b["t_admit"] >= a["t_finish"]
    # the anneals did not wait behind the capped kind
    assert all(r["t_admit"] < r_ns[1]["t_admit"] for r in r_an)
    for job, r in zip(order, res):
        vals, cfg = _oracle(job)
        assert np.array_equal(r["values"], vals), job["kind"]
        assert np.array_equal(r["config"], cfg), job["kind"]
