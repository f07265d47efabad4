#!/usr/bin/env python
"""Benchmark of the GB300 sqaod hot path: dense-graph SQA sweep throughput.

Workload (the large dense single instance of the plain-solver configuration):
N = 4096 spins, m = 256 Trotter replicas, W symmetric uniform[-1, 1] drawn
like sqaod's generate_random_symmetric_W under np.random.seed(0) (diagonal
kept), algorithm = coloring, beta = 50, G = 5.0 * 0.99^k for the 619 steps
k with G > 0.01.  A "step" is one annealOneStep (N * m = 1,048,576 Metropolis
trials).  Each of the K timed units is what the solver runs per field-refresh
period: one sweep launch of 8 consecutive steps, then the field refresh
(--steps-per-launch 1: single-step launches without refresh).  The units start
at positions spread evenly over the 619-step schedule, so the acceptance mix
matches a whole anneal.

  value  : spin-flip trials/s of the device-resident sweep (kernel layer,
           inputs resident in HBM, CUDA events on the launching stream,
           L2 flushed between timed units with a 512 MB write)
  e2e    : the same metric through the solver-handle C ABI with host
           buffers, for one whole anneal as a user runs it: set_qubo (H2D of
           W), seed, prepare, randomize_spin, anneal over the 619-step
           schedule, make_solution, get_E and get_x (D2H)
  roofline: HBM roofline of the sweep kernel (its own launch time, refresh
           excluded): algorithmic bytes per step = A * 4N + 10 N m (A = accepted
           flips counted by the kernel), summed over the launch's steps
  cpu_baseline: the reference CPU coloring annealer (restated with the
           reference's MT19937 and AVX2-order dot), OpenMP on all host cores

--impl reference runs only the CPU reference annealer on the same workload.
Multi-GPU (torchrun): replicas only -- every rank anneals its own instance.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_SPINS, N_TROTTERS = 4096, 256
BETA = 50.0


def schedule():
    G, out = 5.0, []
    while G > 0.01:
        out.append(G)
        G *= 0.99
    return out


def problem(N, seed=0):
    """generate_random_symmetric_W(N, -1, 1) draws under np.random.seed(seed), vectorised."""
    rs = np.random.RandomState(seed)
    iu = np.triu_indices(N)
    W = np.zeros((N, N))
    W[iu] = rs.random_sample(len(iu[0]))
    W = W + np.tril(np.ones((N, N)), -1) * W.T
    return (W * 2.0 - 1.0).astype(np.float32)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def bf16_peak_tflops():
    """Measured dense bf16 tensor rate (burst), else the fallback figure."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


class ClockSampler:
    """Samples the SM clock and clock-event reasons while the timed region runs.

    Reads NVML directly (libnvidia-ml, every 2 ms, on a thread) so that even a
    timed region of a few tens of milliseconds is covered; falls back to
    `nvidia-smi -lms 200`.  Read-only: no clock or other setting is changed.
    """
    # nvmlClocksEventReasons bits
    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown",
               0x4: "sw_power_cap", 0x80: "hw_power_brake_slowdown"}
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu, self.proc, self.path = gpu, None, None
        self.samples, self.stop, self.thread, self.nvml, self.handle = [], False, None, None, None

    def _nvml_open(self):
        try:
            import torch
            nv = ctypes.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() != 0:
                return False
            h = ctypes.c_void_p()
            uuid = getattr(torch.cuda.get_device_properties(self.gpu), "uuid", None)
            ok = False
            if uuid is not None:
                u = str(uuid)
                u = u if u.startswith("GPU-") else "GPU-" + u
                ok = nv.nvmlDeviceGetHandleByUUID(u.encode(), ctypes.byref(h)) == 0
            if not ok:
                cnt = ctypes.c_uint()
                if nv.nvmlDeviceGetCount_v2(ctypes.byref(cnt)) != 0 or cnt.value != 1:
                    return False
                ok = nv.nvmlDeviceGetHandleByIndex_v2(0, ctypes.byref(h)) == 0
            if not ok:
                return False
            self.nvml, self.handle = nv, h
            return True
        except Exception:
            return False

    def _run(self):
        nv, h = self.nvml, self.handle
        mhz, mx, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        get_reasons = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            nv.nvmlDeviceGetCurrentClocksThrottleReasons
        while not self.stop:
            if (nv.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(mhz)) == 0 and
                    nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0 and
                    get_reasons(h, ctypes.byref(rs)) == 0):
                self.samples.append((mhz.value, mx.value, rs.value))
            time.sleep(0.002)

    def __enter__(self):
        if self._nvml_open():
            # the timed region is a tight loop of short host calls: let the
            # sampling thread take the interpreter often
            self.switch = sys.getswitchinterval()
            sys.setswitchinterval(1e-4)
            self.thread = threading.Thread(target=self._run, daemon=True)
            self.thread.start()
            while not self.samples and self.thread.is_alive():
                time.sleep(0.001)
            return self
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                                         stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.thread:
            self.stop = True
            self.thread.join(1.0)
            sys.setswitchinterval(self.switch)
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.thread:
            if not self.samples:
                return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "source": "nvml"}
            reasons = set()
            for _, _, r in self.samples:
                for bit, name in self.REASONS.items():
                    if r & bit:
                        reasons.add(name)
            return {"sm_mhz": statistics.median(s[0] for s in self.samples),
                    "sm_max_mhz": max(s[1] for s in self.samples), "reasons": sorted(reasons),
                    "samples": len(self.samples), "source": "nvml"}
        sm, mx, reasons = [], [], set()
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"),
                                   f[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(name)
            os.unlink(self.path)
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "source": "nvidia-smi"}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm), "source": "nvidia-smi"}


class DenseTask(ctypes.Structure):
    """Mirror of sq103_dense_task (include/sqaod_gb300.h)."""
    _fields_ = [("J", ctypes.c_void_p), ("h", ctypes.c_void_p), ("q", ctypes.c_void_p), ("F", ctypes.c_void_p),
                ("trace", ctypes.c_void_p), ("accepted", ctypes.c_void_p), ("G", ctypes.c_void_p),
                ("beta", ctypes.c_void_p), ("Gs", ctypes.c_float), ("betas", ctypes.c_float),
                ("status", ctypes.c_void_p), ("seed", ctypes.c_uint64), ("step0", ctypes.c_uint32),
                ("N", ctypes.c_int), ("m", ctypes.c_int), ("ldJ", ctypes.c_int), ("algo", ctypes.c_int),
                ("nSteps", ctypes.c_int), ("ws", ctypes.c_void_p), ("wsBytes", ctypes.c_ulonglong),
                ("flags", ctypes.c_int), ("J64", ctypes.c_void_p), ("h64", ctypes.c_void_p)]


def cpu_reference(W, steps, seed=0, min_seconds=0.0, warmup=1, m=N_TROTTERS, n_workers=0):
    """Reference CPU coloring annealer on the host cores (n_workers 0: all of them):
    `warmup` untimed steps, then `steps` annealOneSteps sampled evenly from the
    schedule (repeated until min_seconds have passed); returns (trials/s, cores,
    seconds, steps run)."""
    from oracle import oracle_ctypes as orc
    N = W.shape[0]
    h, J, c = orc.dg_hamiltonian(W)
    a = orc.DenseAnnealerRef(h.astype(np.float32), J.astype(np.float32), float(c), m, n_workers=n_workers)
    a.seed(seed)
    a.randomize_spin()
    sched = schedule()
    idx = np.linspace(0, len(sched) - 1, max(steps, 1)).round().astype(int)
    for i in range(warmup):
        a.anneal_one_step(orc.ALGO_COLORING, sched[i % len(sched)], BETA)
    t0 = time.perf_counter()
    n = 0
    while True:
        for i in idx:
            a.anneal_one_step(orc.ALGO_COLORING, sched[i], BETA)
        n += len(idx)
        if time.perf_counter() - t0 >= min_seconds:
            break
    dt = time.perf_counter() - t0
    return N * m * n / dt, a.workers, dt, n


CPU_LEG_STEPS, CPU_LEG_MIN_SECONDS = 20, 10.0


def cpu_leg(steps, warmup, min_seconds=CPU_LEG_MIN_SECONDS, size=None, workers=0):
    """The reference CPU annealer timed in a fresh process (python bench.py
    --cpu-leg): no torch, no GPU threads beside the OpenMP workers, one thread
    per host core.  The headline line's cpu_baseline and --impl reference both
    use it, with the same sampled schedule positions and minimum duration, so
    the two figures measure the same thing.  Returns (trials/s, cores,
    seconds, steps run)."""
    env = dict(os.environ)
    env["OMP_NUM_THREADS"] = str(os.cpu_count() or 1)
    extra = ["--size", "%d,%d" % size] if size else []
    out = subprocess.run([sys.executable, os.path.abspath(__file__), "--cpu-leg", "--steps", str(steps),
                          "--warmup", str(warmup), "--min-seconds", str(min_seconds),
                          "--cpu-workers", str(workers)] + extra,
                         capture_output=True, text=True, env=env, check=True)
    r = json.loads(out.stdout.strip().splitlines()[-1])
    return r["value"], r["cores"], r["seconds"], r["steps"]


def _sym_uniform(rng, N):
    W = rng.uniform(-1.0, 1.0, (N, N)).astype(np.float32)
    return np.triu(W) + np.triu(W, 1).T


def _log_uniform_int(rng, lo, hi):
    return int(round(float(np.exp(rng.uniform(np.log(lo), np.log(hi))))))


def batched_workload(n_inst=1024, seed=1):
    """1024 uneven dense instances: N log-uniform in [64, 2048], m uniform in
    {8, 16, 32, 64, 128}; instance i draws its couplings from seed 1000 + i."""
    rng = np.random.default_rng(seed)
    return [(_log_uniform_int(rng, 64, 2048), int(rng.choice([8, 16, 32, 64, 128])), 1000 + i)
            for i in range(n_inst)]


def served_stream(rate=200.0, duration=60.0, seed=0):
    """Poisson arrivals; 70 % dense (N log-uniform in [32, 4096]), 30 % bipartite
    (N0, N1 log-uniform in [32, 2048]); m in {16, 64, 256}; request i draws its
    couplings from seed 5000 + i."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t > duration:
            return out
        dense = rng.random() < 0.7
        m = int(rng.choice([16, 64, 256]))
        sizes = ((_log_uniform_int(rng, 32, 4096),) if dense else
                 (_log_uniform_int(rng, 32, 2048), _log_uniform_int(rng, 32, 2048)))
        out.append({"t": t, "dense": dense, "sizes": sizes, "m": m, "seed": 5000 + len(out)})


_POOL = None


def _couplings(req):
    """The request's couplings: a principal submatrix (dense; symmetric) or a block
    (bipartite) of one seeded 4096 x 4096 symmetric uniform[-1, 1] pool, at an
    offset drawn from the request's seed -- deterministic per request, and cheap
    enough to keep up with the arrival rate."""
    global _POOL
    if _POOL is None:
        _POOL = _sym_uniform(np.random.default_rng(12345), 4096)
    rng = np.random.default_rng(req["seed"])
    if req["dense"]:
        N = req["sizes"][0]
        o = int(rng.integers(0, 4096 - N + 1))
        return np.ascontiguousarray(_POOL[o:o + N, o:o + N])
    N0, N1 = req["sizes"]
    o0, o1 = int(rng.integers(0, 4096 - N0 + 1)), int(rng.integers(0, 4096 - N1 + 1))
    return (rng.uniform(-1, 1, N0).astype(np.float32), rng.uniform(-1, 1, N1).astype(np.float32),
            np.ascontiguousarray(_POOL[o1:o1 + N1, o0:o0 + N0]))


def schedule_1000():
    tau = np.exp(np.log(0.01 / 5.0) / 1000)
    return (5.0 * tau ** np.arange(1000)).astype(np.float32)


def _solve_plain(sq, req, G):
    """One request alone on the plain single-instance GPU path; FP64 energies."""
    d = _couplings(req)
    m = req["m"]
    if req["dense"]:
        a = sq.cuda.dense_graph_annealer(d, sq.minimize, n_trotters=m, algorithm="coloring")
    else:
        a = sq.cuda.bipartite_graph_annealer(d[0], d[1], d[2], sq.minimize, n_trotters=m, algorithm="coloring")
    a.seed(req["seed"])
    a.prepare()
    a.randomize_spin()
    a.anneal(G, BETA)
    a.make_solution()
    return a.get_E64()


def _stratified_time(items, cost, solve, n_strata=16, per=3, seed=7):
    """Estimated sequential time of solve() over every item: the items sorted by
    cost, split into n_strata strata of equal count, `per` items drawn at random
    from each and timed; the estimate is sum over strata of (count x mean time),
    with its standard error from the within-stratum spread."""
    order = sorted(range(len(items)), key=lambda i: cost(items[i]))
    rng = np.random.default_rng(seed)
    total, var, timed = 0.0, 0.0, {}
    for st in np.array_split(np.array(order), n_strata):
        if len(st) == 0:
            continue
        pick = rng.choice(st, size=min(per, len(st)), replace=False)
        ts = []
        for i in pick:
            t1 = time.perf_counter()
            timed[int(i)] = solve(items[int(i)])
            ts.append(time.perf_counter() - t1)
        total += len(st) * float(np.mean(ts))
        if len(ts) > 1:
            var += len(st) ** 2 * float(np.var(ts, ddof=1)) / len(ts)
    return total, var ** 0.5, timed


def _request_cost(r):
    return (r["sizes"][0] ** 2 if r["dense"] else r["sizes"][0] * r["sizes"][1]) * r["m"]


def run_served(args, world):
    """C5: the whole seeded stream (Poisson arrivals over the window, 60 s by
    default) submitted at its arrival times and served to the last completion;
    solves/s = requests / makespan.  The plain path's time for the same stream
    (one request after another on the single-instance solvers) is estimated from
    a stratified sample of it, so both rates cover the same request mix."""
    import torch
    import sqaod_gb300 as sq
    from sqaod_gb300.serve import AnnealServer
    reqs = served_stream(duration=args.window)
    G = schedule_1000()
    srv = AnnealServer(budget_bytes=180 << 30, max_slots=args.slots)
    srv.set_large_limit(args.large)
    ticks = 0
    ids, arrival, finish, served_E = {}, {}, {}, {}
    t_gen = t_submit = t_tick = 0.0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    k = 0
    while len(finish) < len(reqs):
        now = time.perf_counter() - t0
        while k < len(reqs) and reqs[k]["t"] <= now:
            ta = time.perf_counter()
            r, d = reqs[k], _couplings(reqs[k])
            tb = time.perf_counter()
            if r["dense"]:
                rid = srv.submit_dense(d, r["m"], G, BETA, sq.minimize, seed=r["seed"])
            else:
                rid = srv.submit_bipartite(d[0], d[1], d[2], r["m"], G, BETA, sq.minimize, seed=r["seed"])
            t_gen += tb - ta
            t_submit += time.perf_counter() - tb
            ids[rid], arrival[rid] = k, r["t"]
            k += 1
        s = srv.stats()
        if s["queued"] == 0 and s["active"] == 0:
            if k < len(reqs):  # idle until the next arrival
                time.sleep(max(0.0, min(0.01, reqs[k]["t"] - (time.perf_counter() - t0))))
            continue
        tc = time.perf_counter()
        nc = srv.tick()
        t_tick += time.perf_counter() - tc
        ticks += 1
        if nc:
            t_now = time.perf_counter() - t0
            for rid in srv.completed():
                finish[rid] = t_now
                E = srv.result(rid)[0]  # released at once; energies kept for the check
                served_E[ids[rid]] = E
    makespan = max(finish.values())
    lat = sorted(finish[r] - arrival[r] for r in finish)
    served = {"solves": len(finish), "makespan_s": makespan, "solves_per_s": len(finish) / makespan,
              "stream_s": args.window, "ticks": ticks, "ms_per_tick": 1000.0 * makespan / max(ticks, 1),
              "host_s": {"generate_couplings": t_gen, "submit": t_submit, "tick": t_tick},
              "p50_s": lat[len(lat) // 2], "p99_s": lat[min(len(lat) - 1, int(0.99 * len(lat)))]}
    del srv
    # the plain path over the same stream, from a stratified sample of it
    t_est, t_se, plain_E = _stratified_time(reqs, _request_cost, lambda r: _solve_plain(sq, r, G),
                                            n_strata=16, per=args.plain_per_stratum)
    plain = {"solves_per_s": len(reqs) / t_est, "seconds_estimated": t_est, "seconds_std_error": t_se,
             "sample": len(plain_E),
             "note": "requests sorted by N^2 m (dense) or N0 N1 m (bipartite), 16 strata of equal count, "
                     "%d timed per stratum on the single-instance solvers (set_qubo, prepare, anneal, "
                     "make_solution, energies); time = sum of count x mean" % args.plain_per_stratum}
    rel = [float(np.max(np.abs(served_E[i] - plain_E[i]) / np.maximum(np.abs(plain_E[i]), 1e-30)))
           for i in plain_E]
    line = {"metric": "served vs plain solves/s (mixed stream)", "value": served["solves_per_s"],
            "unit": "solves/s", "n_gpus": world, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Poisson stream, uniform[-1,1] couplings)",
            "config": {"workload": ("Poisson 200 req/s over %.0f s (%d requests), 70 pct dense N log-uniform "
                                    "[32, 4096], 30 pct bipartite N0/N1 log-uniform [32, 2048], m in {16, 64, 256}, "
                                    "1000-step G 5.0 -> 0.01, beta=50; every request served to completion")
                                   % (args.window, len(reqs)),
                       "slots": args.slots, "large_limit": args.large, "admission_bytes": 180 << 30},
            "served": served, "plain": plain,
            "served_over_plain": served["solves_per_s"] / plain["solves_per_s"],
            "energy_check": {"requests": len(rel), "max_rel_diff": max(rel) if rel else None}}
    print(json.dumps(line), flush=True)


def run_batched(args, world):
    """C4: 1024 uneven instances in one persistent graph-captured launch per
    annealOneStep, against sequential plain solves of a sample of them."""
    import torch
    import sqaod_gb300 as sq
    from sqaod_gb300.batch import DenseBatchAnnealer
    work = batched_workload()
    sched = np.array(schedule(), np.float32)
    steps = len(sched) if args.batch_steps <= 0 else min(args.batch_steps, len(sched))
    G = sched[:steps]
    Ws = [_sym_uniform(np.random.default_rng(seed), N) for N, m, seed in work]
    b = DenseBatchAnnealer()
    t_add = time.perf_counter()
    for (N, m, seed), W in zip(work, Ws):
        b.add(W, m, sq.minimize, seed)
    b.set_schedule(G, BETA)
    if args.multicta_min_n is not None:
        b.set_multicta_min_n(args.multicta_min_n)
    b.prepare()
    torch.cuda.synchronize()
    t_add = time.perf_counter() - t_add
    t_tune = time.perf_counter()
    # trotters per CTA: the one-CTA-per-trotter size limit (default 1024, from whole-run measurements;
    # --autotune-routing times 8 steps per candidate instead); then the staging size, by measurement
    if args.autotune_routing and args.multicta_min_n is None:
        routing = b.autotune_routing(8)
    else:
        routing = 1024 if args.multicta_min_n is None else args.multicta_min_n
    smem = b.autotune(2)
    b.anneal(1, use_graph=True)  # capture + warm up
    b.sync()
    t_tune = time.perf_counter() - t_tune
    b.prepare()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.anneal(steps, use_graph=True)
    b.sync()
    t_batch = time.perf_counter() - t0
    t_out = time.perf_counter()
    for i in range(len(work)):
        b.get_E64(i)
    t_out = time.perf_counter() - t_out
    trials = float(sum(N * m for N, m, _ in work)) * steps
    t_total = t_add + t_batch + t_out
    # plain path: every instance (--plain-sample 0, the default) or an evenly spaced sample
    ns = len(work) if args.plain_sample <= 0 else args.plain_sample
    sample = list(range(0, len(work), max(1, len(work) // ns)))[:ns]
    t_plain, rel = 0.0, []
    for i in sample:
        N, m, seed = work[i]
        W = Ws[i]
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        a = sq.cuda.dense_graph_annealer(W, sq.minimize, n_trotters=m, algorithm="coloring")
        a.seed(seed)
        a.prepare()
        a.randomize_spin()
        a.anneal(G, BETA)
        a.make_solution()
        E = a.get_E64()
        t_plain += time.perf_counter() - t1
        Eb = b.get_E64(i)
        rel.append(float(np.max(np.abs(Eb - E) / np.maximum(np.abs(E), 1e-30))))
        del a
    sample_trials = float(sum(work[i][0] * work[i][1] for i in sample)) * steps
    plain_tps = sample_trials / t_plain
    line = {"metric": "batched vs plain dense anneals (1024 uneven instances)",
            "value": trials / t_batch, "unit": "trials/s", "n_gpus": world, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (W uniform[-1,1] symmetric, seed 1000 + i)",
            "config": {"workload": "1024 dense instances, N log-uniform [64, 2048], m in {8..128}, coloring, "
                                   "beta=50, %d steps of G=5*0.99^k" % steps, "smem_per_cta": smem,
                       "multicta_min_n": routing,
                       "routing": ("autotuned (8 trial steps per candidate 0, 512, 768, 1024, 1400, 2048)"
                                   if args.autotune_routing and args.multicta_min_n is None
                                   else "given" if args.multicta_min_n is not None else "default"),
                       "multicta_instances": b.multicta_count()},
            "batched": {"seconds": t_batch, "solves_per_s": len(work) / t_batch, "setup_s": t_add,
                        "results_s": t_out, "seconds_with_setup": t_total,
                        "solves_per_s_with_setup": len(work) / t_total, "autotune_s": t_tune,
                        "note": "seconds = the annealing launches alone; with_setup adds add()+prepare() of "
                                "all instances and reading every instance's energies (autotune, a one-off, not)"},
            "plain": {"sample": len(sample), "seconds": t_plain, "trials_per_s": plain_tps,
                      "solves_per_s": len(sample) / t_plain if len(sample) == len(work) else None,
                      "solves_per_s_extrapolated": len(work) / (trials / plain_tps),
                      "note": "sequential single-instance solves (set_qubo, prepare, anneal, make_solution, "
                              "energies) of every instance, or of an evenly spaced sample extrapolated by trials"},
            "batched_over_plain": (trials / t_batch) / plain_tps,
            "batched_over_plain_with_setup": (trials / t_total) / plain_tps,
            "energy_check": {"instances": len(rel), "max_rel_diff": max(rel) if rel else None}}
    print(json.dumps(line), flush=True)


def _profiled_traffic(key):
    """DRAM bytes per launch of a kernel, from the ncu capture summarised in profiles/."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(key, {}).get("dram_bytes_per_launch")
    except (OSError, ValueError):
        return None


class BipartiteTask(ctypes.Structure):
    """Mirror of sq103_bipartite_task (include/sqaod_gb300.h)."""
    _fields_ = [("J", ctypes.c_void_p), ("h0", ctypes.c_void_p), ("h1", ctypes.c_void_p), ("q0", ctypes.c_void_p),
                ("q1", ctypes.c_void_p), ("F0", ctypes.c_void_p), ("F1", ctypes.c_void_p),
                ("trace", ctypes.c_void_p), ("accepted", ctypes.c_void_p), ("G", ctypes.c_void_p),
                ("beta", ctypes.c_void_p), ("Gs", ctypes.c_float), ("betas", ctypes.c_float),
                ("seed", ctypes.c_uint64), ("step0", ctypes.c_uint32), ("N0", ctypes.c_int), ("N1", ctypes.c_int),
                ("m", ctypes.c_int), ("algo", ctypes.c_int), ("nSteps", ctypes.c_int),
                ("J64", ctypes.c_void_p), ("h0_64", ctypes.c_void_p), ("h1_64", ctypes.c_void_p),
                ("digits1", ctypes.c_void_p), ("digits0", ctypes.c_void_p), ("spinsBf16", ctypes.c_void_p),
                ("status", ctypes.c_void_p)]


def _timed_steps(stream, flush, K, fn):
    """K calls of fn(i), each bracketed by CUDA events on `stream`, with a
    512 MB write between them (L2 flush, untimed); returns per-call ms."""
    import torch
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    for i in range(K):
        flush.fill_(i & 0xff)
        starts[i].record(stream)
        fn(i)
        ends[i].record(stream)
    torch.cuda.synchronize()
    return [s.elapsed_time(e) for s, e in zip(starts, ends)]


def run_bipartite(args, world):
    """Bipartite SQA coloring, N0 = N1 = 1024, m = 64, beta = 50, the 619-step
    schedule sampled evenly; b0, b1, W iid uniform[-1, 1] under
    np.random.seed(0).  value = trials/s of the device-resident step (kernel
    layer, L2 flushed between steps); the field GEMMs (two per step) are also
    timed alone, since they carry the step's arithmetic."""
    import torch
    import sqaod_gb300 as sq
    from sqaod_gb300 import _lib
    L = _lib.lib()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    N0, N1, m = 1024, 1024, 64
    rs = np.random.RandomState(0)
    b0 = rs.uniform(-1, 1, N0).astype(np.float32)
    b1 = rs.uniform(-1, 1, N1).astype(np.float32)
    W = rs.uniform(-1, 1, (N1, N0)).astype(np.float32)

    def T(a, dt=torch.float32):
        return torch.from_numpy(a).to(dev) if isinstance(a, np.ndarray) else torch.empty(a, dtype=dt, device=dev)

    def P(t):
        return ctypes.c_void_p(t.data_ptr())

    dW, db0, db1 = T(W), T(b0), T(b1)
    J, h0, h1 = T(N1 * N0), T(N0), T(N1)
    c32, c64, scr = T(1), T(1, torch.float64), T(N0 + N1, torch.float64)
    q0, q1 = T(m * N0, torch.int8), T(m * N1, torch.int8)
    F0, F1 = T(m * N0), T(m * N1)
    acc = torch.zeros(1, dtype=torch.int64, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    seed = 1000
    assert L.sq103_bipartite_hamiltonian(P(db0), P(db1), P(dW), N0, N1, 0, P(h0), P(h1), P(J), P(c32), P(c64),
                                         P(scr), sp) == 0
    assert L.sq103_randomize_spins(P(q0), N0, m, ctypes.c_uint64(seed), ctypes.c_uint32(0), 0, sp) == 0
    assert L.sq103_randomize_spins(P(q1), N1, m, ctypes.c_uint64(seed), ctypes.c_uint32(0), 1, sp) == 0
    sched = schedule()
    K, Wm = args.steps, args.warmup
    idx = np.linspace(0, len(sched) - 1, max(K, 1)).round().astype(int)
    step = [1]

    def launch(G):
        t = BipartiteTask(J=J.data_ptr(), h0=h0.data_ptr(), h1=h1.data_ptr(), q0=q0.data_ptr(), q1=q1.data_ptr(),
                          F0=F0.data_ptr(), F1=F1.data_ptr(), trace=None, accepted=acc.data_ptr(), G=None,
                          beta=None, Gs=G, betas=BETA, seed=seed, step0=step[0], N0=N0, N1=N1, m=m, algo=1,
                          nSteps=1)
        rc = L.sq103_bipartite_anneal(ctypes.byref(t), sp)
        if rc != 0:
            raise RuntimeError("sq103_bipartite_anneal failed: %d" % rc)
        step[0] += 1

    for i in range(Wm):
        launch(sched[i % len(sched)])
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        ms = _timed_steps(stream, flush, K, lambda i: launch(sched[idx[i]]))
        gemm_ms = _timed_steps(stream, flush, K, lambda i: (
            L.sq103_bipartite_fields(P(J), N0, N1, P(q0), 1, P(F1), m, sp),
            L.sq103_bipartite_fields(P(J), N0, N1, P(q1), 0, P(F0), m, sp)))
    t_ms = float(np.mean(ms))
    g_ms = float(np.mean(gemm_ms)) / 2
    trials = float(N0 + N1) * m
    value = trials * world / (t_ms / 1e3)
    gemm_flops = 2.0 * m * N0 * N1
    sm_peak_tflops = 152 * 128 * 2 * 2.07e9 / 1e12  # fp32 FMA lanes x max SM clock
    # end to end through the Python solver API, one whole anneal
    G_all = np.array(sched, np.float32)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    a = sq.cuda.bipartite_graph_annealer(b0, b1, W, sq.minimize, n_trotters=m, algorithm="coloring")
    a.seed(seed)
    a.prepare()
    a.randomize_spin()
    a.anneal(G_all, BETA)
    a.make_solution()
    E = a.get_E()
    e2e_s = time.perf_counter() - t0
    nS = len(G_all)
    del a
    # CPU: the restated reference bipartite annealer, a bounded sample of steps
    from oracle import oracle_ctypes as orc
    hh0, hh1, JJ, cc = orc.bg_hamiltonian(b0, b1, W)
    ref = orc.BipartiteAnnealerRef(hh0.astype(np.float32), hh1.astype(np.float32), JJ.astype(np.float32),
                                   float(cc), m, n_workers=0)
    ref.seed(0)
    ref.randomize_spin()
    t1 = time.perf_counter()
    n_cpu = 0
    while time.perf_counter() - t1 < 3.0:
        ref.anneal_one_step(orc.ALGO_COLORING, sched[idx[n_cpu % len(idx)]], BETA)
        n_cpu += 1
    cpu_s = time.perf_counter() - t1
    line = {"metric": "spin-flip trials/s (bipartite SQA coloring, N0=N1=%d m=%d)" % (N0, m), "value": value,
            "unit": "trials/s", "n_gpus": world, "steps": K, "warmup": Wm, "ms_per_step": t_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (b0, b1, W iid uniform[-1,1], np.random.seed(0))",
            "config": {"workload": "bipartite SQA coloring N0=N1=%d m=%d beta=50 G=5*0.99^k (619-step schedule "
                                   "sampled evenly)" % (N0, m), "l2": "flushed between timed steps (512 MB write)"},
            "gpu_launches": K * 6,
            "roofline": {"bound": "fp32 simt", "kernel": "bip_field_kernel (field GEMM, 2 per step)",
                         "achieved": gemm_flops / (g_ms / 1e3) / 1e12, "peak": sm_peak_tflops, "unit": "TFLOP/s",
                         "frac": gemm_flops / (g_ms / 1e3) / 1e12 / sm_peak_tflops,
                         "traffic": _profiled_traffic("bip_field_kernel N0=N1=%d m=%d" % (N0, m)),
                         "peak_source": "nominal fp32 FMA rate at the maximum SM clock",
                         "gemm_ms": g_ms, "gemm_share_of_step": 2 * g_ms / t_ms},
            "e2e": {"value": trials * nS / e2e_s, "unit": "trials/s", "steps": nS, "seconds": e2e_s,
                    "h2d_bytes_per_step": int((W.nbytes + b0.nbytes + b1.nbytes + 2 * G_all.nbytes) / nS),
                    "d2h_bytes_per_step": int((m * (N0 + N1) + 4 * len(E)) / nS), "min_E": float(np.min(E))},
            "cpu_baseline": {"value": trials * n_cpu / cpu_s, "unit": "trials/s", "cores": ref.workers,
                             "kind": "port", "sample": "%d annealOneStep of the same instance, %.1f s" % (n_cpu, cpu_s)},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def bf_problem(N=32, seed=0):
    """W N x N, upper triangle iid integers uniform in [-8, 8] under
    np.random.seed(seed), mirrored; stored fp32."""
    rs = np.random.RandomState(seed)
    U = np.triu(rs.randint(-8, 9, (N, N)))
    return (U + np.triu(U, 1).T).astype(np.float32)


def run_bf(args, world):
    """Dense brute-force search over all 2^32 states of an N = 32 integer
    QUBO (kernel layer: sq103_dense_bf_range over [0, 2^32), min pass and
    argmin collection, then the FP64 re-evaluation of the argmins)."""
    import torch
    import sqaod_gb300 as sq
    from sqaod_gb300 import _lib
    L = _lib.lib()
    L.sq103_bf_workspace_bytes.restype = ctypes.c_size_t
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    N = 32
    W = bf_problem(N)
    dW = torch.from_numpy(W).to(dev)
    ws = torch.empty(int(L.sq103_bf_workspace_bytes(N)), dtype=torch.uint8, device=dev)
    cap = 1 << 16
    cand = torch.empty(cap, dtype=torch.int64, device=dev)
    E64 = torch.empty(cap, dtype=torch.float64, device=dev)
    count = ctypes.c_int()
    Emin = ctypes.c_float()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    nStates = 1 << N

    def search(i):
        rc = L.sq103_dense_bf_range(ctypes.c_void_p(dW.data_ptr()), N, ctypes.c_uint64(0), ctypes.c_uint64(nStates),
                                    ctypes.c_float(0.0), ctypes.c_void_p(ws.data_ptr()),
                                    ctypes.c_void_p(cand.data_ptr()), cap, ctypes.byref(count), ctypes.byref(Emin), sp)
        if rc != 0:
            raise RuntimeError("sq103_dense_bf_range failed: %d" % rc)
        n = min(count.value, cap)
        if n:
            L.sq103_dense_bf_refine(ctypes.c_void_p(dW.data_ptr()), N, ctypes.c_void_p(cand.data_ptr()), n,
                                    ctypes.c_void_p(E64.data_ptr()), sp)

    K, Wm = args.steps, args.warmup
    for i in range(Wm):
        search(i)
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        ms = _timed_steps(stream, flush, K, search)
    t_ms = float(np.mean(ms))
    value = nStates * world / (t_ms / 1e3)
    # the reference formulation's arithmetic per state: the X.W GEMM row plus the row dot (2N^2 + 2N)
    ref_flops = (2.0 * N * N + 2.0 * N) * nStates
    ref_tflops = ref_flops / (t_ms / 1e3) / 1e12
    bf16_peak, bf16_src = bf16_peak_tflops()
    # end to end: the Python searcher (set_qubo uploads W, search, argmins back)
    t0 = time.perf_counter()
    s = sq.cuda.dense_graph_bf_searcher(W, sq.minimize)
    s.search()
    E_api = s.get_E()
    x_api = s.get_x()
    e2e_s = time.perf_counter() - t0
    del s
    # CPU: the restated reference searcher (CPUDenseGraphBFSearcher, all host threads) over the whole
    # N = 28 problem, where the reference times its CPU search; and its X.W tile arithmetic alone
    # on a 2^25-state sample of the N = 32 problem
    from oracle import oracle_ctypes as orc
    W28 = bf_problem(28)
    t1 = time.perf_counter()
    E28, xs28 = orc.dg_bf_search_ref(W28)
    cpu28_s = time.perf_counter() - t1
    tile, n_tiles = 1024, 1 << 15
    t1 = time.perf_counter()
    orc.dg_bf_sweep_tiles(W, 0, tile, n_tiles, 0)
    cpu_s = time.perf_counter() - t1
    line = {"metric": "states/s (dense brute-force search, N=32)", "value": value, "unit": "states/s",
            "n_gpus": world, "steps": K, "warmup": Wm, "ms_per_step": t_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (W 32x32, iid integers uniform[-8, 8] upper triangle mirrored, np.random.seed(0))",
            "config": {"workload": "dense BF N=32, all 2^32 states per step", "l2": "flushed between timed steps",
                       "Emin": float(Emin.value), "argmins": int(count.value)},
            "gpu_launches": K * 5,
            "roofline": {"bound": "tensor", "achieved": ref_tflops, "peak": bf16_peak, "unit": "TFLOP/s",
                         "frac": ref_tflops / bf16_peak, "traffic": None, "peak_source": bf16_src,
                         "note": "achieved = the reference formulation's arithmetic (X.W per tile plus the row "
                                 "dot, 2N^2+2N flops per state) per second; peak = the measured dense bf16 "
                                 "tensor rate, the ceiling of that formulation as a tensor-core GEMM.  This "
                                 "search does not run the GEMM: 2^14-entry tables, about 3 lookups and adds "
                                 "per state, issue-bound; frac > 1 means above the GEMM formulation's ceiling"},
            "e2e": {"value": nStates / e2e_s, "unit": "states/s", "seconds": e2e_s, "h2d_bytes_per_step": W.nbytes,
                    "d2h_bytes_per_step": int(len(E_api) * 4 + np.asarray(x_api).size),
                    "Emin": float(np.min(E_api))},
            "cpu_baseline": {"value": float(1 << 28) / cpu28_s, "unit": "states/s", "cores": os.cpu_count(),
                             "kind": "port",
                             "sample": "the whole N=28 search (2^28 states, W 28x28 integers in [-8, 8] under seed 0) "
                                       "with the restated reference CPU searcher, %.1f s: Emin %g, %d minimisers"
                                       % (cpu28_s, E28, len(xs28)),
                             "tile_arithmetic_states_per_s": tile * n_tiles / cpu_s,
                             "tile_arithmetic_sample": "%d states of the N=32 problem (tiles of %d from x = 0), %.1f s"
                                                       % (tile * n_tiles, tile, cpu_s)},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def run_reference(args, rank):
    if rank != 0:
        return
    W = problem(N_SPINS)
    from oracle import build as ob
    ob.build_oracle()
    ref_kind = "port"
    val, cores, dt, n = cpu_leg(CPU_LEG_STEPS, args.warmup)
    line = {"impl": "reference", "metric": "spin-flip trials/s (dense SQA coloring, N=4096 m=256)",
            "value": val, "unit": "trials/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * dt / max(args.steps, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (sqaod generate_random_symmetric_W, seed 0)",
            "config": {"workload": "dense SQA coloring N=4096 m=256 beta=50 G=5*0.99^k (619-step schedule)",
                       "N": N_SPINS, "m": N_TROTTERS, "algorithm": "coloring"},
            "cpu_baseline": {"value": val, "unit": "trials/s", "cores": cores, "kind": ref_kind,
                             "sample": "%d annealOneSteps (1,048,576 trials each) at %d positions sampled evenly "
                                       "over the 619-step schedule, after %d warm-up steps, %.1f s, in a fresh "
                                       "process" % (n, CPU_LEG_STEPS, args.warmup, dt)},
            "e2e": {"value": val, "unit": "trials/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--size", default="%d,%d" % (N_SPINS, N_TROTTERS),
                    help="N,m of the instance (smaller cases are for profiling captures only)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling captures)")
    ap.add_argument("--steps-per-launch", type=int, default=8, choices=[1, 8],
                    help="sweep mode: annealOneSteps per timed sweep launch (8: one field-refresh period, "
                         "refresh included, as the solver runs them; 1: single-step launches, no refresh)")
    ap.add_argument("--mode", default="sweep", choices=["sweep", "batched", "served", "bipartite", "bf"],
                    help="sweep: the headline dense sweep; batched: 1024 uneven instances; served: mixed stream; "
                         "bipartite: N0=N1=1024 m=64 sweep; bf: dense brute force N=32")
    ap.add_argument("--window", type=float, default=60.0, help="served mode: seconds of Poisson arrivals")
    ap.add_argument("--plain-per-stratum", type=int, default=3,
                    help="served mode: plain solves timed per stratum of the stream (16 strata)")
    ap.add_argument("--slots", type=int, default=512, help="served mode: concurrent instances per kind")
    ap.add_argument("--large", type=int, default=64,
                    help="served mode: concurrent large instances (dense ones step together in packed launches)")
    ap.add_argument("--check", type=int, default=16, help="served mode: requests compared with the plain path")
    ap.add_argument("--batch-steps", type=int, default=0, help="batched mode: steps (0 = the whole schedule)")
    ap.add_argument("--plain-sample", type=int, default=0,
                    help="batched mode: instances solved on the plain path (0: all of them)")
    ap.add_argument("--autotune-routing", action="store_true",
                    help="batched mode: choose the one-CTA-per-trotter size limit by timing 8 steps per candidate")
    ap.add_argument("--multicta-min-n", type=int, default=None,
                    help="batched mode: instances of at least this N take the one-CTA-per-trotter sweep (default 1024)")
    ap.add_argument("--cpu-leg", action="store_true", help="internal: time the CPU reference annealer alone")
    ap.add_argument("--min-seconds", type=float, default=CPU_LEG_MIN_SECONDS, help="--cpu-leg: minimum duration")
    ap.add_argument("--cpu-workers", type=int, default=0, help="--cpu-leg: host threads (0: all)")
    args = ap.parse_args()

    if args.cpu_leg:
        Nc, mc = (int(v) for v in args.size.split(","))
        val, cores, dt, n = cpu_reference(problem(Nc), args.steps, min_seconds=args.min_seconds, m=mc,
                                          n_workers=args.cpu_workers,
                                          warmup=args.warmup)
        print(json.dumps({"value": val, "cores": cores, "seconds": dt, "steps": n}), flush=True)
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return

    import torch
    torch.cuda.set_device(local)
    if args.mode != "sweep":
        if rank == 0:
            {"batched": run_batched, "served": run_served, "bipartite": run_bipartite, "bf": run_bf}[args.mode](
                args, world)
        return
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    import sqaod_gb300 as sq
    from sqaod_gb300 import _lib
    L = _lib.lib()
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    dev = torch.device("cuda", local)
    N, m = (int(v) for v in args.size.split(","))
    W = problem(N)

    def P(t):
        return ctypes.c_void_p(t.data_ptr())

    # -------- device-resident sweep (kernel layer)
    dW = torch.from_numpy(W).to(dev)
    dJ = torch.empty((N, N), dtype=torch.float32, device=dev)
    dh = torch.empty(N, dtype=torch.float32, device=dev)
    c32 = torch.empty(1, dtype=torch.float32, device=dev)
    c64 = torch.empty(1, dtype=torch.float64, device=dev)
    scratch = torch.empty(N, dtype=torch.float64, device=dev)
    q = torch.empty(m * N, dtype=torch.int8, device=dev)
    F = torch.empty(m * N, dtype=torch.float32, device=dev)
    acc = torch.zeros(1, dtype=torch.int64, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    seed = 1000 + rank
    assert L.sq103_dense_hamiltonian(P(dW), N, N, 0, P(dh), P(dJ), N, P(c32), P(c64), P(scratch), sp) == 0
    assert L.sq103_randomize_spins(P(q), N, m, ctypes.c_uint64(seed), ctypes.c_uint32(0), 0, sp) == 0
    # the refresh the solver runs: tensor-core digit contraction for N >= 1024, else SIMT
    L.sq103_tc_digits_bytes.restype = ctypes.c_ulonglong
    L.sq103_tc_spins_bytes.restype = ctypes.c_ulonglong
    use_tc = bool(L.sq103_dense_refresh_uses_tc(N))
    digits = torch.empty(int(L.sq103_tc_digits_bytes(N, N)) if use_tc else 1, dtype=torch.uint8, device=dev)
    abf = torch.empty(int(L.sq103_tc_spins_bytes(m, N)) if use_tc else 1, dtype=torch.uint8, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    if use_tc:
        assert L.sq103_tc_make_digits(P(dJ), N, N, N, 0, P(digits), sp) == 0
    dig_p = P(digits) if use_tc else None

    def refresh_fields():
        return L.sq103_dense_refresh(P(dJ), N, dig_p, P(abf), P(q), P(F), N, m, P(status), sp)

    assert refresh_fields() == 0
    sched = schedule()
    K, Wm = args.steps, args.warmup
    spl = args.steps_per_launch
    # timed iteration i: spl annealOneSteps from schedule position s0[i] (spread
    # evenly over the schedule) in one sweep launch, then -- for spl = 8, one
    # field-refresh period -- the refresh the solver runs after every 8 steps
    s0 = np.linspace(0, len(sched) - spl, max(K, 1)).round().astype(int)
    dG = torch.tensor(sched, dtype=torch.float32, device=dev)
    dB = torch.full_like(dG, BETA)

    L.sq103_dense_ws_bytes.restype = ctypes.c_ulonglong
    ws_bytes = int(L.sq103_dense_ws_bytes(N, m, spl))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    multi = bool(L.sq103_dense_multicta_ok(N, m, 1))
    refresh = spl == 8

    def launch(pos, step):
        t = DenseTask(J=dJ.data_ptr(), h=dh.data_ptr(), q=q.data_ptr(), F=F.data_ptr(), trace=None,
                      accepted=acc.data_ptr(), G=dG.data_ptr() + 4 * pos, beta=dB.data_ptr() + 4 * pos, Gs=0.0,
                      betas=BETA, status=status.data_ptr(), seed=seed, step0=step, N=N, m=m, ldJ=N, algo=1,
                      nSteps=spl, ws=ws.data_ptr(), wsBytes=ws_bytes, flags=0)
        rc = L.sq103_dense_anneal(ctypes.byref(t), sp)
        if rc != 0:
            raise RuntimeError("sq103_dense_anneal failed: %d" % rc)

    def do_refresh():
        if refresh and refresh_fields() != 0:
            raise RuntimeError("sq103_dense_refresh failed")

    step = 1
    for i in range(Wm):
        launch((i * spl) % (len(sched) - spl + 1), step)
        do_refresh()
        step += spl
    torch.cuda.synchronize()
    acc_hist = torch.zeros(K + 1, dtype=torch.int64, device=dev)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    mids = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        acc_hist[0].copy_(acc[0])
        for i in range(K):
            flush.fill_(i & 0xff)  # L2 flush between timed iterations (untimed)
            starts[i].record(stream)
            launch(int(s0[i]), step)
            mids[i].record(stream)
            acc_hist[i + 1].copy_(acc[0])
            do_refresh()
            ends[i].record(stream)
            step += spl
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    if int(status.item()) != 0:
        raise RuntimeError("sweep kernel reported device status %d" % int(status.item()))
    t_ms = float(sum(a.elapsed_time(b) for a, b in zip(starts, ends)))
    sweep_ms = float(sum(a.elapsed_time(b) for a, b in zip(starts, mids)))
    # replicas: every rank ran its own instance; the job rate is all ranks'
    # trials over the slowest rank's time
    from sqaod_gb300.shard import replica_throughput
    trials = float(N) * m * K * spl
    value, t_ms = replica_throughput(t_ms, trials, device=dev)
    accepted = (acc_hist[1:] - acc_hist[:-1]).cpu().numpy().astype(np.float64)  # per launch
    alg_bytes = accepted * 4.0 * N + 10.0 * N * m * spl                          # per launch
    achieved_gbs = float(alg_bytes.sum()) / (sweep_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    # the field refresh of each timed unit (launched after the sweep, timed by the same events):
    # 2 N^2 m algorithmic flops; the tensor-core path issues four digit contractions of that size
    refresh_info = None
    if refresh:
        r_ms = float(sum(a.elapsed_time(b) for a, b in zip(mids, ends))) / K
        flops = 2.0 * N * N * m
        refresh_info = {"kernel": "tc_digit_gemm (tcgen05, 4 bf16 digit planes, exact)" if use_tc
                        else "field_gemm_kernel (fp32 SIMT)", "ms_per_launch": r_ms,
                        "algorithmic_tflops": flops / (r_ms / 1e3) / 1e12,
                        "mma_tflops": (4.0 if use_tc else 1.0) * flops / (r_ms / 1e3) / 1e12}

    # -------- end to end through the solver-handle C ABI with host buffers: one
    # whole anneal of the 619-step schedule, as a user runs it (set_qubo uploads W,
    # anneal runs the schedule, make_solution / get_E / get_x bring the result back)
    e2e = None
    if not args.no_e2e:
        Wh = np.ascontiguousarray(W)
        G_all = np.array(sched, np.float32)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ann = sq.cuda.dense_graph_annealer(Wh, sq.minimize, n_trotters=m, algorithm="coloring")
        ann.seed(seed)
        ann.prepare()
        ann.randomize_spin()
        t1 = time.perf_counter()
        ann.anneal(G_all, BETA)
        t2 = time.perf_counter()
        ann.make_solution()
        E = ann.get_E()
        x = ann.get_x()
        e2e_s = time.perf_counter() - t0
        phases = {"setup_s": t1 - t0, "anneal_s": t2 - t1, "solution_s": e2e_s - (t2 - t0)}
        nS = len(G_all)
        e2e = {"value": float(N) * m * nS / e2e_s, "unit": "trials/s",
               "h2d_bytes_per_step": int((Wh.nbytes + G_all.nbytes * 2) / nS),
               "d2h_bytes_per_step": int((m * N + 4 * len(E)) / nS),
               "steps": nS, "seconds": e2e_s, "phases": phases, "min_E": float(np.min(E))}
        del ann, x

    cpu = None
    if rank == 0 and not args.no_cpu_baseline and (N, m) == (N_SPINS, N_TROTTERS):
        val, cores, dt, n = cpu_leg(CPU_LEG_STEPS, args.warmup)
        cpu = {"value": val, "unit": "trials/s", "cores": cores, "kind": "port",
               "sample": "%d annealOneSteps (1,048,576 trials each) at %d positions sampled evenly over the "
                         "619-step schedule, after %d warm-up steps, %.1f s, in a fresh process"
                         % (n, CPU_LEG_STEPS, args.warmup, dt)}
    elif rank == 0 and not args.no_cpu_baseline:
        # other sizes (C1 is the reference's own CPU case): the faster of all host threads and one
        # thread -- at small N the per-step parallel regions can cost more than they share
        runs = [cpu_leg(CPU_LEG_STEPS, args.warmup, min_seconds=5.0, size=(N, m), workers=w) for w in (0, 1)]
        val, cores, dt, n = max(runs, key=lambda r: r[0])
        cpu = {"value": val, "unit": "trials/s", "cores": cores, "kind": "port",
               "sample": "%d annealOneSteps (%d trials each) at %d positions sampled evenly over the 619-step "
                         "schedule, %.1f s, in a fresh process; the faster of all host threads (%.3g trials/s) "
                         "and one thread (%.3g trials/s)" % (n, N * m, CPU_LEG_STEPS, dt, runs[0][0], runs[1][0])}

    if rank == 0:
        traffic = _profiled_traffic("dense_sweep_multi N=%d m=%d steps=%d" % (N, m, spl))
        line = {"metric": "spin-flip trials/s (dense SQA coloring, N=%d m=%d)" % (N, m), "value": value,
                "unit": "trials/s", "n_gpus": world, "steps": K * spl, "warmup": Wm * spl,
                "ms_per_step": t_ms / (K * spl),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (sqaod generate_random_symmetric_W(%d, -1, 1), np.random.seed(0))" % N,
                "config": {"workload": "dense SQA coloring N=%d m=%d beta=50 G=5*0.99^k (619-step " % (N, m) +
                                       "schedule sampled evenly over the timed steps)",
                           "N": N, "m": m, "algorithm": "coloring",
                           "timed_unit": ("%d annealOneSteps in one sweep launch + the field refresh the solver "
                                          "runs every 8 steps" % spl) if refresh else
                                         ("%d annealOneStep(s) per sweep launch, no refresh" % spl),
                           "l2": "flushed between timed units (512 MB write)",
                           "kernel": "one CTA per trotter (cooperative)" if multi else "one CTA per instance",
                           "parallelism": "replicas" if world > 1 else "single instance"},
                "e2e": e2e, "gpu_launches": K * (1 + ((2 if use_tc else 1) if refresh else 0)),
                "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": peak, "unit": "GB/s",
                             "frac": achieved_gbs / peak, "traffic": traffic, "peak_source": peak_kind,
                             "algorithmic_bytes_per_launch": float(alg_bytes.mean()),
                             "steps_per_launch": spl, "sweep_ms_per_launch": sweep_ms / K,
                             "accepted_per_step": float(accepted.mean()) / spl,
                             "refresh": refresh_info},
                "cpu_baseline": cpu, "clocks": clk.summary(), "wall_s": wall}
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
