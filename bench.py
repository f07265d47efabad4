#!/usr/bin/env python
"""Benchmark of the GB300 sqaod hot path: dense-graph SQA sweep throughput.

Workload (the large dense single instance of the plain-solver configuration):
N = 4096 spins, m = 256 Trotter replicas, W symmetric uniform[-1, 1] drawn
like sqaod's generate_random_symmetric_W under np.random.seed(0) (diagonal
kept), algorithm = coloring, beta = 50, G = 5.0 * 0.99^k for the 619 steps
k with G > 0.01.  A "step" is one annealOneStep (N * m = 1,048,576 Metropolis
trials).  The K timed steps sample the 619-step schedule evenly, so the
acceptance mix matches a whole anneal.

  value  : spin-flip trials/s of the device-resident sweep (kernel layer,
           inputs resident in HBM, CUDA events on the launching stream,
           L2 flushed between timed steps with a 512 MB write)
  e2e    : the same metric through the solver-handle C ABI with host
           buffers, for one whole anneal as a user runs it: set_qubo (H2D of
           W), seed, prepare, randomize_spin, anneal over the 619-step
           schedule, make_solution, get_E and get_x (D2H)
  roofline: HBM roofline of the sweep kernel: algorithmic bytes per launch
           = A * 4N + 10 N m (A = accepted flips counted by the kernel)
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
                ("flags", ctypes.c_int)]


def cpu_reference(W, steps, seed=0):
    """Reference CPU coloring annealer on the host cores; returns (trials/s, cores, seconds)."""
    from oracle import oracle_ctypes as orc
    N = W.shape[0]
    h, J, c = orc.dg_hamiltonian(W)
    a = orc.DenseAnnealerRef(h.astype(np.float32), J.astype(np.float32), float(c), N_TROTTERS, n_workers=0)
    a.seed(seed)
    a.randomize_spin()
    sched = schedule()
    idx = np.linspace(0, len(sched) - 1, max(steps, 1)).round().astype(int)
    t0 = time.perf_counter()
    for i in idx:
        a.anneal_one_step(orc.ALGO_COLORING, sched[i], BETA)
    dt = time.perf_counter() - t0
    return N * N_TROTTERS * len(idx) / dt, a.workers, dt


def run_reference(args, rank):
    if rank != 0:
        return
    W = problem(N_SPINS)
    from oracle import build as ob
    ob.build_oracle()
    ref_kind = "port"
    val, cores, dt = cpu_reference(W, args.steps)
    line = {"impl": "reference", "metric": "spin-flip trials/s (dense SQA coloring, N=4096 m=256)",
            "value": val, "unit": "trials/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * dt / max(args.steps, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (sqaod generate_random_symmetric_W, seed 0)",
            "config": {"workload": "dense SQA coloring N=4096 m=256 beta=50 G=5*0.99^k (619-step schedule)",
                       "N": N_SPINS, "m": N_TROTTERS, "algorithm": "coloring"},
            "cpu_baseline": {"value": val, "unit": "trials/s", "cores": cores, "kind": ref_kind,
                             "sample": "%d annealOneStep of the 619-step schedule (sampled evenly)" % args.steps},
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
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return

    import torch
    torch.cuda.set_device(local)
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
    assert L.sq103_dense_field_refresh(P(dJ), N, P(q), P(F), N, m, sp) == 0
    sched = schedule()
    K, Wm = args.steps, args.warmup
    idx = np.linspace(0, len(sched) - 1, max(K, 1)).round().astype(int)

    L.sq103_dense_ws_bytes.restype = ctypes.c_ulonglong
    ws_bytes = int(L.sq103_dense_ws_bytes(N, m, 1))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    multi = bool(L.sq103_dense_multicta_ok(N, m, 1))

    def launch(G, step):
        t = DenseTask(J=dJ.data_ptr(), h=dh.data_ptr(), q=q.data_ptr(), F=F.data_ptr(), trace=None,
                      accepted=acc.data_ptr(), G=None, beta=None, Gs=G, betas=BETA, status=status.data_ptr(),
                      seed=seed, step0=step, N=N, m=m, ldJ=N, algo=1, nSteps=1, ws=ws.data_ptr(),
                      wsBytes=ws_bytes, flags=0)
        rc = L.sq103_dense_anneal(ctypes.byref(t), sp)
        if rc != 0:
            raise RuntimeError("sq103_dense_anneal failed: %d" % rc)

    step = 1
    for i in range(Wm):
        launch(sched[i % len(sched)], step)
        step += 1
    torch.cuda.synchronize()
    acc_hist = torch.zeros(K + 1, dtype=torch.int64, device=dev)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        acc_hist[0].copy_(acc[0])
        for i in range(K):
            flush.fill_(i & 0xff)  # L2 flush between timed steps (untimed)
            starts[i].record(stream)
            launch(sched[idx[i]], step)
            ends[i].record(stream)
            step += 1
            acc_hist[i + 1].copy_(acc[0])
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    if int(status.item()) != 0:
        raise RuntimeError("sweep kernel reported device status %d" % int(status.item()))
    kernel_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    t_ms = float(sum(kernel_ms))
    if dist:
        tt = torch.tensor([t_ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_ms = float(tt.item())
    accepted = (acc_hist[1:] - acc_hist[:-1]).cpu().numpy().astype(np.float64)
    trials = float(N) * m * K
    value = trials * world / (t_ms / 1e3)
    alg_bytes = accepted * 4.0 * N + 10.0 * N * m
    achieved_gbs = float(alg_bytes.sum()) / (t_ms / 1e3) / 1e9
    peak, peak_kind = peaks()

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
        val, cores, dt = cpu_reference(W, 1)
        cpu = {"value": val, "unit": "trials/s", "cores": cores, "kind": "port",
               "sample": "1 annealOneStep (1,048,576 trials) at G=5.0 of the same instance, %.1f s" % dt}

    if rank == 0:
        traffic = None
        try:
            with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
                traffic = json.load(f).get("dense_sweep_multi N=%d m=%d" % (N, m), {}).get("dram_bytes_per_launch")
        except (OSError, ValueError):
            traffic = None
        line = {"metric": "spin-flip trials/s (dense SQA coloring, N=%d m=%d)" % (N, m), "value": value,
                "unit": "trials/s", "n_gpus": world, "steps": K, "warmup": Wm, "ms_per_step": t_ms / K,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (sqaod generate_random_symmetric_W(%d, -1, 1), np.random.seed(0))" % N,
                "config": {"workload": "dense SQA coloring N=%d m=%d beta=50 G=5*0.99^k (619-step " % (N, m) +
                                       "schedule sampled evenly over the timed steps)",
                           "N": N, "m": m, "algorithm": "coloring", "l2": "flushed between timed steps (512 MB write)",
                           "kernel": "one CTA per trotter (cooperative)" if multi else "one CTA per instance",
                           "parallelism": "replicas" if world > 1 else "single instance"},
                "e2e": e2e, "gpu_launches": K,
                "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": peak, "unit": "GB/s",
                             "frac": achieved_gbs / peak, "traffic": traffic, "peak_source": peak_kind,
                             "algorithmic_bytes_per_launch": float(alg_bytes.mean()),
                             "accepted_per_step": float(accepted.mean())},
                "cpu_baseline": cpu, "clocks": clk.summary(), "wall_s": wall}
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
