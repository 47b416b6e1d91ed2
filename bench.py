"""Benchmark: batched Metropolis swap trials on GB300 (one JSON line).

Workload (the batched-replica configuration): 1024 independent bcc replicas,
lattice edge L drawn per replica from {8, 12, 16, 24} (1024-27648 sites),
4 equiatomic species, 6 coordination shells, V symmetric 4x4 per shell drawn
uniform[-0.05, 0.05] eV from a fixed seed (converted to Ry), temperatures
log-spaced 100-3000 K (one per replica), mt19937ar seed 110179 + 11 r per
replica, random initial configurations drawn by initial_setup on the device.
One step = `--sweeps-per-step` sweeps (N_r trials each) of every replica in
one launch; 50 steps of 10 sweeps make the 500-sweep run.

Reported:
  value        trials/s with all state resident in HBM (device-timed)
  e2e          trials/s through the C ABI with host buffers: every step
               moves all replicas' configurations host->device, runs, and
               moves them back (plus the accept counts), one call
               (brawl_batch_metropolis_host) whose kernels read and write
               the pinned host buffer in place
  roofline     algorithmic bytes per launch / kernel time, against the
               measured HBM copy bandwidth
  cpu_baseline the CPU oracle (a restatement of the reference's serial
               Fortran, which needs gfortran/netCDF absent here) on all host
               cores, on a bounded sample of the same replicas
  plain_gpu    the one-chain-per-launch GPU path on a sample of replicas

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

# More hardware work queues than the default 8: the serving leg keeps long
# rounds of kernels in flight on a few streams, and jobs' set-up and
# read-back on their own streams must not queue behind them.  Read when the
# CUDA context is created, so it is set before torch is imported.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

RY_TO_EV = 13.605693122
K_B_IN_RY = 8.167333262e-5 / 13.605693122990
METRIC = "swap trials/s"
WORKLOAD = "batched Metropolis: 1024 bcc replicas, L in {8,12,16,24}, 4 species, 6 shells"


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def make_workload(n_rep: int = 1024, seed: int = 20260, rank: int = 0):
    rng = np.random.default_rng(seed)
    Ls = rng.choice(np.array([8, 12, 16, 24]), size=n_rep)
    ns, nsh = 4, 6
    V = np.zeros((ns, ns, nsh))
    for sh in range(nsh):
        a = rng.uniform(-0.05, 0.05, size=(ns, ns))
        V[:, :, sh] = np.triu(a) + np.triu(a, 1).T
    V /= RY_TO_EV
    r = np.arange(n_rep)
    T = 100.0 * 30.0 ** (r / max(n_rep - 1, 1))
    seeds = 110179 + 11 * (r + rank * n_rep)
    conc = np.array([0.0, 0.25, 0.25, 0.25, 0.25])
    return dict(L=Ls, V=V, T=T, seeds=seeds, conc=conc, ns=ns, nsh=nsh)


def n_sites(L: int) -> int:
    return 2 * L * L * L


# ---------------------------------------------------------------------------
# CPU side (oracle port): one process per core, each owning one replica
# ---------------------------------------------------------------------------
def _cpu_worker(conn, replica: int, wl: dict):
    from oracle import oracle as O
    L = int(wl["L"][replica])
    mod = O.OracleModel("bcc", L, L, L, wl["V"])
    rng = O.OracleRng(int(wl["seeds"][replica]))
    cfg, _ = mod.initial_setup(rng, wl["conc"])
    beta = 1.0 / (float(wl["T"][replica]) * K_B_IN_RY)
    conn.send("ready")
    while True:
        msg = conn.recv()
        if msg is None:
            break
        t0 = time.perf_counter()
        acc, _ = mod.mc_run(cfg, rng, beta, int(msg))
        conn.send((int(msg), time.perf_counter() - t0))
    conn.close()


class CpuPool:
    """Started with 'spawn' before any CUDA call."""

    def __init__(self, n_procs: int, wl: dict):
        ctx = mp.get_context("spawn")
        self.conns, self.procs = [], []
        # replicas spread over the four lattice sizes
        order = np.argsort(wl["L"], kind="stable")
        for k in range(n_procs):
            replica = int(order[(k * len(order)) // n_procs])
            a, b = ctx.Pipe()
            p = ctx.Process(target=_cpu_worker, args=(b, replica, wl), daemon=True)
            p.start()
            self.conns.append(a)
            self.procs.append(p)
        for c in self.conns:
            assert c.recv() == "ready"

    def run(self, trials_each: int):
        t0 = time.perf_counter()
        for c in self.conns:
            c.send(trials_each)
        res = [c.recv() for c in self.conns]
        wall = time.perf_counter() - t0
        return sum(r[0] for r in res), wall

    def close(self):
        for c in self.conns:
            try:
                c.send(None)
            except Exception:
                pass
        for p in self.procs:
            p.join(timeout=5)


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_calibrate(pool: CpuPool, seconds: float) -> int:
    n, wall = pool.run(20000)
    per = max(wall, 1e-6) / 20000
    return max(20000, int(seconds / per))


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.lines = []
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(device_index)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def smem_bandwidth_gbs() -> float | None:
    """The device's shared-memory bandwidth (GB/s) from the library's own
    streaming-load kernel, measured outside every timed region."""
    import ctypes as C
    import brawl_gb300 as B
    v = C.c_double(0.0)
    try:
        rc = B.load().brawl_smem_bandwidth(C.byref(v))
    except Exception:
        return None
    return v.value / 1e9 if rc == 0 and v.value > 0 else None


def committed_smem() -> dict | None:
    """Shared-memory bytes and issue activity of the Metropolis kernel from
    the committed ncu summary (profiles/metropolis_batched_smem.json)."""
    p = os.path.join(ROOT, "profiles", "metropolis_batched_smem.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


def roofline_object(achieved_gbs, smem_peak, peaks, traffic, alg_per_step, trials_per_s) -> dict:
    """The Metropolis kernel against the ceiling that bounds it: its bytes
    are served from shared memory (DRAM traffic per launch is the lattices'
    staging only), so the peak is the measured shared-memory bandwidth; the
    HBM copy rate is given beside it."""
    out = {"bound": "smem", "achieved": achieved_gbs, "unit": "GB/s",
           "peak": smem_peak, "frac": (achieved_gbs / smem_peak) if smem_peak else None,
           "peak_source": "measured in this run (brawl_smem_bandwidth)",
           "traffic": traffic, "algorithmic_bytes_per_step": alg_per_step,
           "hbm": {"peak": peaks["hbm_gbs"], "frac": achieved_gbs / peaks["hbm_gbs"],
                   "peak_source": peaks["source"]},
           "note": "latency-bound sequential chains (one warp per chain, a dependent chain of "
                   "shared loads, a warp reduction and a decision per trial); achieved = the "
                   "canonical algorithmic bytes per trial over the kernel's event time"}
    cs = committed_smem()
    if cs:
        out["ncu"] = cs
        # the shared-memory bytes the kernel moves per trial (ncu wavefronts
        # of the committed capture) at this run's rate, against the ceiling
        bpt = cs["smem_wavefronts_per_trial"] * cs["bytes_per_wavefront"]
        gbs = bpt * trials_per_s / 1e9
        out["smem_traffic"] = {"bytes_per_trial": bpt, "achieved": gbs, "unit": "GB/s",
                               "frac": (gbs / smem_peak) if smem_peak else None}
    return out


def committed_traffic() -> dict | None:
    """DRAM traffic per launch of the Metropolis kernel on the 1024-replica
    workload, from the committed ncu summary
    (profiles/metropolis_batched_traffic.json), if present."""
    p = os.path.join(ROOT, "profiles", "metropolis_batched_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


class UtilSampler:
    """utilization.gpu (the fraction of time a kernel ran) every 200 ms."""

    def __init__(self, device_index: int):
        self.vals = []
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=utilization.gpu", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(device_index)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            try:
                self.vals.append((time.perf_counter(), float(line.strip())))
            except ValueError:
                pass

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        return self.vals


def _mean_util(samples, t_lo, t_hi):
    v = [u for t, u in samples if t_lo <= t <= t_hi]
    return float(np.mean(v)) / 100.0 if v else None


def _serve_latency(args, SV, dev, rate: float, n_jobs: int) -> dict:
    """Poisson arrivals of the seeded mixed stream at `rate` jobs/s; latency
    = finish - submit per job, p50/p99 overall and by kind, the device's
    busy fraction while jobs arrive."""
    jobs = SV.stream_jobs(n_jobs, master_seed=424242, L_range=(6, args.serve_L_max),
                          sweeps_range=(100, args.serve_sweeps_max))
    rng = np.random.default_rng(99)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, len(jobs)))
    util = UtilSampler(dev)
    with SV.Server() as srv:
        ids = []
        t0 = time.perf_counter()
        for job, t in zip(jobs, arrivals):
            dt = t0 + t - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            ids.append(srv.submit(job))
        t_arrived = time.perf_counter()
        res = []
        for i in ids:
            try:
                res.append(srv.wait(i, timeout=900.0))
            except Exception as e:   # a job that did not end in time counts as failed
                res.append({"status": getattr(e, "code", -1), "t_submit": 0.0, "t_admit": 0.0,
                            "t_finish": 0.0, "trials": 0})
        makespan = time.perf_counter() - t0
        stats = srv.stats()
        prof = srv.profile()
    samples = util.stop()
    ok = [r for r in res if r["status"] == 0]
    failed = {}
    for job, r in zip(jobs, res):
        if r["status"] != 0:
            key = f'{job["kind"]}:{r["status"]}'
            failed[key] = failed.get(key, 0) + 1
    lat = np.array([r["t_finish"] - r["t_submit"] for r in ok])
    queue = np.array([r["t_admit"] - r["t_submit"] for r in ok])
    by_kind = {}
    for job, r in zip(jobs, res):
        if r["status"] == 0:
            by_kind.setdefault(job["kind"], []).append(r["t_finish"] - r["t_submit"])
    trials = sum(SV.job_trials(j) for j, r in zip(jobs, res) if r["status"] == 0 and j["kind"] != "ns")
    ns_steps = sum(int(r["trials"]) for j, r in zip(jobs, res) if r["status"] == 0 and j["kind"] == "ns")
    counts = {k: sum(1 for j in jobs if j["kind"] == k) for k in ("anneal", "wl", "ns")}
    return {
        "stream": f"{len(jobs)} jobs (of the 10^4 of the full stream) of the seeded mixed stream: "
                  f"fcc/bcc, L in [6,{args.serve_L_max}], 2-5 species (Dirichlet composition), "
                  f"2-6 shells, V uniform +-0.05 eV; anneal 100-{args.serve_sweeps_max} sweeps over "
                  "4 temperatures, WL window (4 walkers, 256 bins, 20 one-sweep calls), NS run "
                  "(64 walkers, 100 iterations of one-sweep walks)",
        "jobs_by_kind": counts,
        "arrivals": f"Poisson, {rate} jobs/s over {arrivals[-1]:.0f} s",
        "jobs_ok": len(ok), "jobs_failed": failed,
        "p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
        "p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
        "p50_queue_s": float(np.percentile(queue, 50)) if len(queue) else None,
        "p99_queue_s": float(np.percentile(queue, 99)) if len(queue) else None,
        "p50_by_kind_s": {k: float(np.percentile(v, 50)) for k, v in by_kind.items()},
        "p99_by_kind_s": {k: float(np.percentile(v, 99)) for k, v in by_kind.items()},
        "makespan_s": makespan,
        "trials_per_s": (trials + ns_steps) / makespan,
        "gpu_busy_while_arriving": _mean_util(samples, t0, t_arrived),
        "rounds": stats["rounds"],
        "busy_s_by_pipeline": {k: round(v["busy_s"], 2) for k, v in prof.items()},
    }


def serving_leg(args) -> dict:
    """The serving stream through the continuous-batching loop
    (brawl_serve_*), on the mixed workload's ranges: fcc/bcc, L in [6, 32],
    2-5 species, 2-6 shells, anneals of 100-2000 sweeps, Wang-Landau windows
    and nested-sampling runs.  Two phases.
    latency: Poisson arrivals at args.serve_rate jobs/s (below capacity),
      latency = finish - submit per job, p50/p99 overall and by kind, the
      device's busy fraction while jobs arrive;
    saturation: arrivals far above capacity for args.serve_sat_seconds;
      throughput = work the scheduler handed out per second once the resident
      set has filled (trials; Wang-Landau summed over walkers; nested
      sampling walk steps), and the busy fraction over the same window."""
    from brawl_gb300 import serving as SV
    dev = torch_device_index()
    out = {}
    # ---- latency phase
    out["latency"] = _serve_latency(args, SV, dev, args.serve_rate, args.serve_jobs)
    # ---- optional latency curve: the same stream at other arrival rates
    rates = [float(x) for x in args.serve_rate_sweep.split(",") if x.strip()]
    if rates:
        curve = []
        for r in rates:
            L = _serve_latency(args, SV, dev, r, args.serve_sweep_jobs)
            curve.append({"rate_jobs_per_s": r, "jobs": L["jobs_ok"], "p50_s": L["p50_s"], "p99_s": L["p99_s"],
                          "p50_by_kind_s": L["p50_by_kind_s"], "p99_by_kind_s": L["p99_by_kind_s"],
                          "p99_queue_s": L["p99_queue_s"], "trials_per_s": L["trials_per_s"],
                          "gpu_busy_while_arriving": L["gpu_busy_while_arriving"]})
        out["latency_curve"] = curve
    # ---- saturation phases: the mixed stream, then its anneal jobs alone
    rng = np.random.default_rng(99)
    n_sat = int(args.serve_sat_rate * args.serve_sat_seconds)
    for key, kinds in (("saturation", None), ("saturation_anneal_only", ("anneal",))):
        if n_sat <= 0:
            break
        jobs = SV.stream_jobs(n_sat if kinds is None else 3 * n_sat, master_seed=525252,
                              L_range=(6, args.serve_L_max), sweeps_range=(100, args.serve_sweeps_max))
        if kinds is not None:
            jobs = [j for j in jobs if j["kind"] in kinds]
        arrivals = np.cumsum(rng.exponential(1.0 / args.serve_sat_rate, len(jobs)))
        util = UtilSampler(dev)
        series = []
        with SV.Server() as srv:
            t0 = time.perf_counter()
            k = 0
            t_next = t0
            while time.perf_counter() - t0 < args.serve_sat_seconds:
                now = time.perf_counter() - t0
                while k < len(jobs) and arrivals[k] <= now:
                    srv.submit(jobs[k])
                    k += 1
                if time.perf_counter() >= t_next:
                    p = srv.profile()
                    st = srv.stats()
                    series.append((time.perf_counter(), sum(v["work"] for v in p.values()),
                                   st["resident"], st["queued"]))
                    t_next += 1.0
                time.sleep(0.005)
            # the window: from a third of the phase to its end
        samples = util.stop()
        lo = series[len(series) // 3]
        hi = series[-1]
        out[key] = {
            "jobs": "the mixed stream" if kinds is None else "the mixed stream's anneal jobs",
            "arrivals": f"Poisson, {args.serve_sat_rate} jobs/s for {args.serve_sat_seconds} s "
                        "(far above capacity: the queue grows)",
            "window_s": hi[0] - lo[0],
            "trials_per_s": (hi[1] - lo[1]) / (hi[0] - lo[0]),
            "resident_jobs": [lo[2], hi[2]],
            "queued_jobs": [lo[3], hi[3]],
            "gpu_busy": _mean_util(samples, lo[0], hi[0]),
            "note": "work handed out by the scheduler per second: swap trials of anneal chains "
                    "and Wang-Landau walkers, nested-sampling walk steps at n_steps per iteration",
        }
    return out


def torch_device_index() -> int:
    import torch
    return torch.cuda.current_device() if torch.cuda.is_available() else 0


# neighbours within the first k shells (k = 1, 2, ...)
Z_CUMULATIVE = {"bcc": (8, 14, 26, 50, 58, 64, 88, 112, 136, 168), "fcc": (12, 18, 42, 54, 78, 86)}


def _wl_cpu(setup, V, cfg, edges, bins, period, seconds: float = 3.0) -> dict:
    """The oracle's sweeps() for one walker on one host core, a bounded
    sample of about `seconds`."""
    from oracle import oracle as O
    mod = O.OracleModel("bcc", *setup.n, V)
    cfg = np.ascontiguousarray(cfg, dtype=np.int8).copy()
    rng = O.OracleRng(110179)
    lng = np.zeros(bins)
    hist = np.zeros(bins)
    e = mod.total_energy(cfg)
    n = 20000
    t0 = time.perf_counter()
    _, e, _ = mod.wl_sweep(cfg, rng, edges, lng, hist, e, bins, 1, bins, n, 1.0, period)
    est = n / max(1e-6, time.perf_counter() - t0)
    n2 = max(n, int(est * seconds))
    t0 = time.perf_counter()
    mod.wl_sweep(cfg, rng, edges, lng, hist, e, bins, 1, bins, n2, 1.0, period)
    dt = time.perf_counter() - t0
    return {"value": n2 / dt, "unit": "trials/s", "cores": 1, "kind": "port",
            "sample": f"one walker, {n2} trials of sweeps() on the oracle, {dt:.1f} s"}


def _ns_cpu(V, conc, seconds: float = 3.0) -> dict:
    """The oracle's nested-sampling run (same shape) on one host core: the
    iterations' walks after the walkers are set up, a bounded sample."""
    from oracle import oracle as O
    mod = O.OracleModel("fcc", 6, 6, 6, V)
    t0 = time.perf_counter()
    mod.ns_run(O.OracleRng(7), conc, None, 1024, 2000, 1)
    t1 = time.perf_counter()
    mod.ns_run(O.OracleRng(7), conc, None, 1024, 2000, 3)
    t2 = time.perf_counter()
    per_iter = max(1e-6, (t2 - t1 - (t1 - t0)) / 2.0)
    m = int(min(400, max(3, seconds / per_iter)))
    t3 = time.perf_counter()
    mod.ns_run(O.OracleRng(7), conc, None, 1024, 2000, m + 1)
    dt = time.perf_counter() - t3 - (t1 - t0)
    # fewer than K/2 iterations: every walk is exactly 2000 steps
    return {"value": m * 2000 / dt, "unit": "steps/s", "cores": 1, "kind": "port",
            "sample": f"K = 1024, {m} iterations of 2000-step walks on the oracle "
                      f"(set-up and first iteration subtracted), {dt:.1f} s"}


def walker_legs(args) -> dict:
    """Wang-Landau and nested-sampling throughput at the shapes of the
    reference's WL and NS workloads (seeded synthetic inputs).  Both APIs
    block until the device is done, so each leg is timed on the host around
    its calls, with the device synchronised on both sides.

    * WL: bcc 12^3, 4 species, 4 shells, V uniform +-0.05 eV, 128 walkers
      (32 groups of 4 averaged together) from random configurations, each
      in a 1000-bin window around those configurations' energies, wl_f = 1;
      sweeps() calls of 10^4 trials per walker (the exchange interval).
    * NS: fcc 6^3, 5 species, 3 shells, V uniform +-0.08 eV, K = 1024
      walkers, 2000-step walks; a bounded sample of iterations.
    """
    import torch
    import brawl_gb300 as B
    from brawl_gb300 import serving as SV
    out = {}
    if "wl" in args.walker_legs:
        rng = np.random.default_rng(20261)
        ns, nsh, L, nw, bins = 4, 4, 12, 128, 1000
        V = SV.symmetric_V(rng, ns, nsh, 0.05)
        setup = B.Setup("bcc", L, L, L, ns, nsh)
        conc = np.array([0.0] + [0.25] * 4)
        tmp = B.Batch([dict(setup=setup, V=V, seed=110179 + 11 * k, beta=0.0, species_concentrations=conc)
                       for k in range(nw)])
        cfgs = [tmp.config(k) for k in range(nw)]
        E = tmp.total_energy()
        tmp.close()
        c, hw = float(E.mean()), float(np.abs(E - E.mean()).max() * 1.2 + 1e-3)
        edges = (c - hw) + np.arange(bins + 1) * (2 * hw / bins)
        walkers = [dict(setup=setup, V=V, seed=110179 + 11 * k, config=cfgs[k], start_idx=1, end_idx=bins,
                        window=k // 4) for k in range(nw)]
        wl = B.WangLandauWalkers(walkers, edges)
        n, calls = 10000, args.wl_calls
        period = int(0.02 * float(np.float32(setup.n_atoms)))
        wl.sweeps(n, 1.0, period)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(calls):
            wl.sweeps(n, 1.0, period)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        c0 = {}
        for w in range(nw):
            for k, v in wl.counters(w).items():
                c0[k] = c0.get(k, 0) + int(v)
        wl.close()
        # the timed calls' share of the counters (the warm-up call is the other)
        cnt = {k: v * calls // (calls + 1) for k, v in c0.items()}
        z = Z_CUMULATIVE["bcc"][nsh - 1]
        # algorithmic bytes: every trial reads its two species and the pair's
        # z neighbours with one V row each (2 + 2z + 16z), an evaluated trial
        # the same again after the swap (16z), 4 bytes per stream word
        alg = cnt["trials"] * (2 + 18 * z) + cnt["evaluated"] * 16 * z + 4 * cnt["draws"]
        peaks = measured_peaks()
        out["wang_landau"] = {
            "metric": "WL trials/s", "value": nw * n * calls / dt, "unit": "trials/s",
            "workload": "bcc 12^3, 4 species, 4 shells, 128 walkers, 1000-bin windows, "
                        f"{calls} sweeps() calls of 10^4 trials per walker",
            "us_per_trial_per_walker": dt / (n * calls) * 1e6,
            "accepted_fraction": cnt["accepted"] / max(1, cnt["trials"]),
            "exact_now_fraction": cnt["exact_path"] / max(1, cnt["evaluated"]),
            "roofline": {"bound": "latency", "achieved": alg / dt / 1e9, "peak": peaks["hbm_gbs"],
                         "peak_kind": "HBM copy, for scale", "unit": "GB/s",
                         "frac": alg / dt / 1e9 / peaks["hbm_gbs"],
                         "note": "algorithmic bytes over host-timed calls; each walker is one warp's "
                                 "dependent chain of trials (lattice and tables in shared memory), so "
                                 "neither HBM nor shared-memory bandwidth bounds it"},
            "cpu_baseline": _wl_cpu(setup, V, cfgs[0], edges, bins, period),
        }
        if args.wl_seconds > 0:
            out["wang_landau"]["windows_run"] = _wl_windows_run(args, setup, V, conc)
    if "ns" in args.walker_legs:
        rng = np.random.default_rng(20263)
        ns, nsh = 5, 3
        V = SV.symmetric_V(rng, ns, nsh, 0.08)
        setup = B.Setup("fcc", 6, 6, 6, ns, nsh)
        conc = np.array([0.0] + [0.2] * 5)
        run = B.NestedSampling([dict(setup=setup, V=V, seed=7, n_walkers=1024, n_steps=2000,
                                     species_concentrations=conc)])
        run.iterate(5)
        c0 = run.counters(0)["trials"]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        run.iterate(args.ns_iterations)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        cnt1 = run.counters(0)
        steps = cnt1["trials"] - c0
        run.close()
        # independent runs side by side (one per SM): the replica-parallel
        # throughput of the same kernel
        n_runs = args.ns_runs
        ens = B.NestedSampling([dict(setup=setup, V=V, seed=7 + 11 * r, n_walkers=1024, n_steps=2000,
                                     species_concentrations=conc) for r in range(n_runs)])
        ens.iterate(2)
        e0 = sum(ens.counters(r)["trials"] for r in range(n_runs))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ens.iterate(args.ns_iterations // 5 or 1)
        torch.cuda.synchronize()
        edt = time.perf_counter() - t0
        esteps = sum(ens.counters(r)["trials"] for r in range(n_runs)) - e0
        ens.close()
        z = Z_CUMULATIVE["fcc"][nsh - 1]
        # every step evaluates its pair before and after (2 + 2z + 32z bytes);
        # the stream words drawn for the iteration's steps, 4 bytes each
        draws = cnt1["draws"] * steps // max(1, cnt1["trials"])
        alg = steps * (2 + 34 * z) + 4 * draws
        peaks = measured_peaks()
        out["nested_sampling"] = {
            "metric": "NS walk steps/s", "value": steps / dt, "unit": "steps/s",
            "workload": f"fcc 6^3, 5 species, 3 shells, K = 1024, 2000-step walks, "
                        f"{args.ns_iterations} iterations after 5",
            "iterations_per_s": args.ns_iterations / dt,
            "independent_runs": {"runs": n_runs, "value": esteps / edt, "unit": "steps/s",
                                 "sample": f"{args.ns_iterations // 5 or 1} iterations of every run "
                                           "after 2, one launch"},
            "roofline": {"bound": "latency", "achieved": alg / dt / 1e9, "peak": peaks["hbm_gbs"],
                         "peak_kind": "HBM copy, for scale", "unit": "GB/s",
                         "frac": alg / dt / 1e9 / peaks["hbm_gbs"],
                         "note": "algorithmic bytes over host-timed calls; one sequential run of "
                                 "dependent walk steps, its flushes' FP64 sums spread over four warps"},
            "cpu_baseline": _ns_cpu(V, conc),
        }
    return out


def _wl_windows_run(args, setup, V, conc) -> dict:
    """The Wang-Landau workload's own layout through the driver
    (brawl_gb300.wang_landau): 32000 bins split by divide_range into 32
    windows of 1000 bins, each extended downwards by create_overlap (bin
    overlap 0.25), 4 walkers per window (128), flatness 0.8, ln f from 1,
    sweeps() calls of 10^4 trials per walker with replica exchange between
    adjacent windows after every call, the in-window averages and
    dos_combine at every halving.  The energy range (meV/atom) runs from the
    mean energy of a pilot anneal (8 chains, 300 K, 300 sweeps) to the mean
    of 128 random configurations (the energies the temperature search that
    places the walkers in their windows can reach).  The run is bounded by args.wl_seconds; the
    time to ln f < 1e-6 (20 halvings) is extrapolated from the halvings
    reached: the sweeps() calls per halving are fitted as c_k = a r^k on
    the measured ones (least squares on log c_k) and the remaining
    halvings cost their fitted calls at the run's seconds per call."""
    import torch
    import brawl_gb300 as B
    from brawl_gb300 import inputs as I
    from brawl_gb300 import wang_landau as WLD
    N = setup.n_atoms
    pilot = B.Batch([dict(setup=setup, V=V, seed=31 + k, beta=1.0 / (300.0 * B.K_B_IN_RY),
                          species_concentrations=conc) for k in range(8)])
    pilot.metropolis(300 * N)
    e_lo = float(pilot.total_energy().mean())
    pilot.close()
    rnd = B.Batch([dict(setup=setup, V=V, seed=1000 + k, beta=0.0, species_concentrations=conc)
                   for k in range(128)])
    e_hi = float(rnd.total_energy().mean())
    rnd.close()
    to_mev = B.RY_TO_EV * 1000.0 / N
    p = I.WLParams(mc_sweeps=0, bins=32000, num_windows=32, bin_overlap=float(np.float32(0.25)),
                   tolerance=1e-6, flatness=float(np.float32(0.8)), wl_f=1.0,
                   energy_min=float(np.float32(e_lo * to_mev)), energy_max=float(np.float32(e_hi * to_mev)))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = WLD.wang_landau(setup, V, conc, p, walkers_per_window=4, trials_per_call=10_000,
                          deadline_s=args.wl_seconds, burn_in="temperature")
    torch.cuda.synchronize()
    total = time.perf_counter() - t0
    rec = res["record"]
    calls = res["calls"]
    loop_s = args.wl_seconds if not rec or rec[-1]["wl_f"] > p.tolerance else rec[-1]["seconds"]
    per_call = loop_s / max(1, calls)
    c_k, prev = [], 0
    for r in rec:
        c_k.append(r["calls"] - prev)
        prev = r["calls"]
    est = None
    if len(c_k) >= 2:
        k = np.arange(1, len(c_k) + 1)
        b, a = np.polyfit(k, np.log(np.maximum(c_k, 1)), 1)
        fitted = [float(np.exp(a + b * kk)) for kk in range(len(c_k) + 1, 21)]
        est = loop_s + (sum(fitted) - (calls - prev) if fitted else 0.0) * per_call
    return {
        "layout": "bcc 12^3, 4 species, 4 shells; 32000 bins, 32 windows (divide_range, "
                  "create_overlap 0.25), 4 walkers each; exchange after every 10^4-trial call",
        "energy_range_mev_per_atom": [p.energy_min, p.energy_max],
        "seconds": total, "loop_seconds": loop_s, "calls": calls,
        "trials_per_s": 128 * 10_000 * calls / loop_s,
        "ln_f_reached": rec[-1]["wl_f"] if rec else 1.0,
        "calls_per_halving": c_k,
        "seconds_at_halving": [round(float(r["seconds"]), 2) for r in rec],
        "seconds_to_ln_f_1e-6_extrapolated": est,
        "extrapolation": "calls per halving fitted as a*r^k on the measured halvings; "
                         "the halvings up to 2^-20 < 1e-6 at the run's seconds per call",
    }


def anneal_leg(args) -> dict:
    """The reference's own serial case: simulated annealing of one fcc 8^3
    chain (2048 sites, 2 species 1024/1024, 2 shells, V uniform +-0.05 eV),
    T = 1500 -> 300 K in 13 steps of 1000 sweeps, the energy sampled every
    sweep, ASRO off, static seed of rank 0.  The GPU runs all of it through
    the annealing driver (one chain: a latency-bound sequence of trials);
    the oracle a bounded sample of its first temperatures on one host core."""
    import torch
    import brawl_gb300 as B
    from brawl_gb300 import inputs as I
    from brawl_gb300 import metropolis as M
    from brawl_gb300 import serving as SV
    from oracle import oracle as O
    rng = np.random.default_rng(20260)
    V = SV.symmetric_V(rng, 2, 2, 0.05)
    setup = B.Setup("fcc", 8, 8, 8, 2, 2)
    N = setup.n_atoms
    conc = np.array([0.0, 0.5, 0.5])
    nums = np.array([1024, 1024], dtype=np.int64)

    def params(T_steps):
        return I.MetropolisParams(mode="simulated_annealing", n_mc_steps=1000 * N, n_sample_steps=N,
                                  calculate_energies=True, calculate_asro=False, n_sample_steps_asro=N,
                                  n_sample_steps_trajectory=N, T=1500.0, T_steps=T_steps, delta_T=-100.0)
    ch = B.Chain(setup, V)
    ch.f90_init_genrand(0, 0)
    ch.initial_setup(conc, nums)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = M.simulated_annealing(ch, params(13), 2, record_configs=False)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    trials = 13 * 1000 * N
    mod = O.OracleModel("fcc", 8, 8, 8, V)
    r = O.OracleRng(O.lib().bo_static_seed(0))
    cfg, _ = mod.initial_setup(r, conc, nums)
    m2 = params(args.anneal_cpu_temperatures)
    ap = dict(T=m2.T, delta_T=m2.delta_T, T_steps=m2.T_steps, n_mc_steps=m2.n_mc_steps, n_burn_in_steps=0,
              n_sample_steps=m2.n_sample_steps, n_sample_steps_asro=m2.n_sample_steps_asro,
              n_sample_steps_alro=0, n_sample_steps_trajectory=m2.n_sample_steps_trajectory, burn_in=0,
              burn_in_start=0, calculate_energies=1, calculate_asro=0, nbr_swap=0, wc_range=2)
    t1 = time.perf_counter()
    ref = mod.anneal(cfg, r, ap)
    cdt = time.perf_counter() - t1
    k = args.anneal_cpu_temperatures
    same = bool(np.array_equal(ref["energies_of_T"][:k], out["energies_of_T"][:k]))
    return {"metric": "swap trials/s (one chain)", "value": trials / dt, "unit": "trials/s",
            "workload": "simulated annealing, fcc 8^3, 2 species, 2 shells, T 1500 -> 300 K in 13 steps "
                        "of 1000 sweeps, energy every sweep, one chain",
            "seconds": dt,
            "cpu_baseline": {"value": k * 1000 * N / cdt, "unit": "trials/s", "cores": 1, "kind": "port",
                             "sample": f"the first {k} temperatures on the oracle, {cdt:.1f} s"},
            "energies_match_oracle": same}


def max_over_ranks(x: float, world: int, device=None) -> float:
    """The largest x over the ranks (the job's time is its slowest rank's)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args, world, rank):
    """The reference arm: the CPU implementation of the path (the oracle port
    of the reference's serial Fortran) on all host cores."""
    if rank != 0:
        return 0
    wl = make_workload(args.replicas)
    cores = host_cores()
    pool = CpuPool(cores, wl)
    trials_each = cpu_calibrate(pool, 2.0)
    for _ in range(args.warmup):
        pool.run(trials_each)
    tot, wall = 0, 0.0
    for _ in range(args.steps):
        n, w = pool.run(trials_each)
        tot += n
        wall += w
    pool.close()
    v = tot / wall
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "trials/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * wall / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int8+f64",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "replicas": args.replicas,
                   "step": f"{cores} replicas x {trials_each} trials, one process per core"},
        "cpu_baseline": {"value": v, "unit": "trials/s", "cores": cores, "kind": "port",
                         "sample": f"{cores} replicas (spread over L) x {trials_each} trials per step"},
        "e2e": {"value": v, "unit": "trials/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--replicas", type=int, default=1024)
    ap.add_argument("--sweeps-per-step", type=int, default=10)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--serve-jobs", type=int, default=600)
    ap.add_argument("--serve-rate", type=float, default=10.0)
    ap.add_argument("--serve-L-max", type=int, default=32)
    ap.add_argument("--serve-sweeps-max", type=int, default=2000)
    ap.add_argument("--serve-sat-rate", type=float, default=250.0)
    ap.add_argument("--serve-rate-sweep", default="",
                    help="comma-separated arrival rates (jobs/s) for a latency curve (empty: none)")
    ap.add_argument("--serve-sweep-jobs", type=int, default=300)
    ap.add_argument("--serve-sat-seconds", type=float, default=45.0)
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--walker-legs", default="wl,ns",
                    help="Wang-Landau / nested-sampling legs to run (wl, ns; empty for none)")
    ap.add_argument("--walker-legs-only", action="store_true",
                    help="run only the walker legs and print their JSON")
    ap.add_argument("--wl-calls", type=int, default=5)
    ap.add_argument("--wl-seconds", type=float, default=60.0,
                    help="budget of the Wang-Landau run on the workload's window layout (0: skip)")
    ap.add_argument("--ns-iterations", type=int, default=50)
    ap.add_argument("--anneal-leg", type=int, default=1, help="time the one-chain annealing case (0: skip)")
    ap.add_argument("--anneal-cpu-temperatures", type=int, default=3)
    ap.add_argument("--ns-runs", type=int, default=152,
                    help="independent nested-sampling runs of the replica-parallel measurement")
    ap.add_argument("--speculation", type=int, default=0,
                    help="trials per speculative round of the Metropolis kernel (0: library default)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank)

    args.walker_legs = [x for x in args.walker_legs.split(",") if x]
    if args.walker_legs_only:
        import torch
        torch.cuda.set_device(local)
        print(json.dumps(walker_legs(args)))
        return 0

    wl = make_workload(args.replicas, rank=rank)
    # CPU baseline workers first: spawned before any CUDA call
    pool = None
    if rank == 0 and world == 1 and not args.no_cpu:
        pool = CpuPool(host_cores(), wl)

    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import brawl_gb300 as B

    setup_by_L = {L: B.Setup("bcc", L, L, L, wl["ns"], wl["nsh"]) for L in (8, 12, 16, 24)}
    chains = []
    for r in range(args.replicas):
        L = int(wl["L"][r])
        chains.append(dict(setup=setup_by_L[L], V=wl["V"], seed=int(wl["seeds"][r]),
                           beta=1.0 / (float(wl["T"][r]) * K_B_IN_RY),
                           species_concentrations=wl["conc"]))
    batch = B.Batch(chains)
    sites = np.array([n_sites(int(L)) for L in wl["L"]], dtype=np.int64)
    trials = sites * args.sweeps_per_step
    trials_per_step = int(trials.sum())
    if args.speculation:
        batch.set_speculation(args.speculation)
        cta_shape = {"trials_per_round": args.speculation, "picked_by": "--speculation"}
    else:
        # the CTA shape by measurement, before the warm-up and outside every
        # timed region: per class of chains (lattice, L, species, shells),
        # each in its own launch with its own shared memory, the trials per
        # round from one sweep of every chain at each depth, from the same
        # state, which the library restores after each try
        try:
            tuned = batch.autotune_classes(sites, max_depth=4)
            cta_shape = {"picked_by": "autotune per chain class (whole-batch time, median of 3)",
                         "tuning_sample": "one sweep of every chain", **tuned}
        except Exception as exc:  # keep one warp per chain and say why
            batch.set_speculation(1)
            cta_shape = {"trials_per_round": 1, "picked_by": "default", "autotune_error": str(exc)[:200]}

    stream = torch.cuda.Stream()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def step_device():
        batch.metropolis_async(trials, stream.cuda_stream)

    for _ in range(args.warmup):
        with torch.cuda.stream(stream):
            step_device()
        batch.sync()
    c0 = batch.counters()

    # ---- device-resident timed region -------------------------------------
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    t_wall0 = time.perf_counter()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()                      # inputs < L2: flush between steps
            starts[k].record(stream)
            step_device()
            ends[k].record(stream)
    stream.synchronize()
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    batch.sync()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    dev_s = sum(step_ms) / 1000.0
    c1 = batch.counters()
    dev_s = max_over_ranks(dev_s, world, "cuda")
    d = (c1 - c0).sum(axis=0)
    T_all, T_eval, draws = int(d[0]), int(d[1]), int(d[2])
    assert T_all == trials_per_step * args.steps, (T_all, trials_per_step * args.steps)
    value = world * T_all / dev_s

    # roofline: algorithmic bytes B = 2 T_all + (2 + 2z + 32z) T_eval + 4 D
    z = 64
    alg_bytes = 2 * T_all + (2 + 2 * z + 32 * z) * T_eval + 4 * draws
    achieved_gbs = alg_bytes / dev_s / 1e9
    peaks = measured_peaks()
    smem_peak = smem_bandwidth_gbs()
    traffic = None
    tr = committed_traffic()
    if tr and tr.get("dram_bytes_per_launch") and args.replicas == 1024:
        traffic = float(tr["dram_bytes_per_launch"])     # one launch per step

    # ---- end to end through the C ABI with host buffers -------------------
    grid_bytes = batch.grid_bytes
    pinned = torch.empty(grid_bytes, dtype=torch.int8, pin_memory=True)
    host_grids = pinned.numpy()
    batch.get_configs(host_grids)
    e2e_steps = max(3, args.steps // 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        # every replica's config from the pinned host buffer, the run, the
        # configs back into it and the accept counts: one call, the kernels
        # reading and writing the page-locked buffer in place (NVLink-C2C)
        acc = batch.metropolis_host(host_grids, trials)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, "cuda")
    e2e_value = world * trials_per_step * e2e_steps / e2e_s
    h2d = grid_bytes + 8 * args.replicas
    d2h = grid_bytes + 8 * args.replicas * 9

    # ---- plain one-chain-per-launch path on a sample -----------------------
    sample = []
    for L in (8, 12, 16, 24):
        idx = np.nonzero(wl["L"] == L)[0]
        sample += [int(i) for i in idx[:2]]
    plain_chains = [chains[i] for i in sample]
    pb = B.Batch(plain_chains)
    ptrials = np.array([n_sites(int(wl["L"][i])) for i in sample], dtype=np.int64)
    pb.metropolis_serial(ptrials // 10)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pb.metropolis_serial(ptrials)
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    plain_value = float(ptrials.sum()) / plain_s
    pb.close()

    # ---- CPU baseline (oracle port) ------------------------------------------
    cpu = None
    if pool is not None:
        each = cpu_calibrate(pool, args.cpu_seconds)
        n, w = pool.run(each)
        cores = len(pool.conns)
        pool.close()
        cpu = {"value": n / w, "unit": "trials/s", "cores": cores, "kind": "port",
               "sample": f"{cores} replicas of the workload (spread over L), {each} trials each, "
                         f"one process per core, {w:.1f} s"}

    serving = None
    if rank == 0 and world == 1 and not args.no_serve and args.serve_jobs > 0:
        serving = serving_leg(args)
    walkers = walker_legs(args) if rank == 0 and world == 1 and args.walker_legs else {}
    anneal = anneal_leg(args) if rank == 0 and world == 1 and args.anneal_leg else None

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "trials/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int8+f64",
            "data": "synthetic (seeded replicas, V and temperatures)",
            "config": {"workload": WORKLOAD, "replicas": args.replicas,
                       "sweeps_per_step": args.sweeps_per_step,
                       "trials_per_step": trials_per_step,
                       "l2": "flushed between steps (256 MiB write)",
                       "parallelism": f"replicas x{world}", "cta_shape": cta_shape},
            "e2e": {"value": e2e_value, "unit": "trials/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": e2e_steps},
            "roofline": roofline_object(achieved_gbs, smem_peak, peaks, traffic,
                                        alg_bytes / args.steps, T_all / dev_s),
            "cpu_baseline": cpu,
            "plain_gpu": {"value": plain_value, "unit": "trials/s",
                          "sample": f"{len(sample)} replicas, 1 sweep each, one launch per replica"},
            "batched_over_plain": value / plain_value,
            "serving": serving,
            "wang_landau": walkers.get("wang_landau"),
            "nested_sampling": walkers.get("nested_sampling"),
            "anneal_one_chain": anneal,
            "clocks": clk,
            # one launch per chain class per step
            "gpu_launches": args.steps * max(1, len(cta_shape.get("classes", [])) or 1),
            "counters": {"trials": T_all, "evaluated": T_eval, "draws": draws,
                         "accepted": int(d[3]), "exp_tests": int(d[4]),
                         "exact_path": int(d[5]), "exp_fp64": int(d[6]), "exp_cr": int(d[7])},
            "wall_s_timed_region": t_wall,
        }
        print(json.dumps(line))
    batch.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
