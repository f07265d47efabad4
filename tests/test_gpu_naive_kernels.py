"""The naive sweeps (dense naive; bipartite naive and sa_naive) through the
kernel layer of the C ABI (sq103_dense_anneal / sq103_bipartite_anneal with
algo 0 / 2), replayed step by step against the FP64 host replay of the same
Philox stream.  The annealers select algorithms as the reference's CUDA
annealers do (naive runs coloring), so these kernels are reached here only."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MARGIN_TOL = 1e-6


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    import bench
    import sqaod_gb300 as sq
    from sqaod_gb300 import _lib
    L = _lib.lib()
    L.sq103_dense_ws_bytes.restype = ctypes.c_ulonglong
    return torch, bench, sq, L


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _sym(rng, N):
    W = rng.uniform(-1, 1, (N, N))
    return (np.triu(W) + np.triu(W, 1).T).astype(np.float32)


@pytest.mark.parametrize("N,m", [(48, 8), (37, 7), (64, 2)])
def test_dense_naive_kernel_replays_fp64(env, orc, N, m):
    torch, bench, sq, L = env
    dev = torch.device("cuda", 0)
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(N * 100 + m)
    h, J, c = sq.cuda.dense_graph_annealer(_sym(rng, N), n_trotters=m).get_hamiltonian()
    dJ = torch.from_numpy(np.ascontiguousarray(J, np.float32)).to(dev)
    dh = torch.from_numpy(np.ascontiguousarray(h, np.float32)).to(dev)
    q = torch.empty(m * N, dtype=torch.int8, device=dev)
    F = torch.empty(m * N, dtype=torch.float32, device=dev)
    nwords = (N * m + 31) // 32
    trace = torch.zeros(nwords, dtype=torch.int32, device=dev)
    acc = torch.zeros(1, dtype=torch.int64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    ws_bytes = int(L.sq103_dense_ws_bytes(N, m, 1))
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    seed = 1234 + N
    assert L.sq103_randomize_spins(_p(q), N, m, ctypes.c_uint64(seed), ctypes.c_uint32(0), 0, sp) == 0
    assert L.sq103_dense_field_refresh(_p(dJ), N, _p(q), _p(F), N, m, sp) == 0
    torch.cuda.synchronize()
    qh = q.cpu().numpy().reshape(m, N)
    assert np.array_equal(qh, orc.gpu_randomize(seed, 0, 0, m, N))
    for step, (G, beta) in enumerate([(3.0, 10.0), (1.0, 10.0), (0.3, 20.0), (0.05, 50.0)], start=1):
        trace.zero_()
        t = bench.DenseTask(J=dJ.data_ptr(), h=dh.data_ptr(), q=q.data_ptr(), F=F.data_ptr(),
                            trace=trace.data_ptr(), accepted=acc.data_ptr(), G=None, beta=None, Gs=G, betas=beta,
                            status=status.data_ptr(), seed=seed, step0=step, N=N, m=m, ldJ=N, algo=0, nSteps=1,
                            ws=ws.data_ptr(), wsBytes=ws_bytes, flags=0)
        assert L.sq103_dense_anneal(ctypes.byref(t), sp) == 0
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        tr = trace.cpu().numpy().view(np.uint32)
        q_host, st = orc.dg_replay(h, J, m, orc.ALGO_NAIVE, seed, step, G, beta, qh, tr, MARGIN_TOL)
        qh = q.cpu().numpy().reshape(m, N)
        assert np.array_equal(qh, q_host), "device state diverged from the replayed trace"
        assert st["n_trials"] == N * m
        assert st["n_mismatch"] == st["n_mismatch_small"], st


@pytest.mark.parametrize("algo", ["naive", "sa_naive"])
@pytest.mark.parametrize("N0,N1,m", [(40, 24, 6), (17, 33, 5)])
def test_bipartite_naive_kernels_replay_fp64(env, orc, algo, N0, N1, m):
    torch, bench, sq, L = env
    dev = torch.device("cuda", 0)
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(N0 * 7 + N1 + m)
    b0, b1 = rng.uniform(-1, 1, N0).astype(np.float32), rng.uniform(-1, 1, N1).astype(np.float32)
    W = rng.uniform(-1, 1, (N1, N0)).astype(np.float32)
    h0, h1, J, c = sq.cuda.bipartite_graph_annealer(b0, b1, W, n_trotters=m).get_hamiltonian()
    T = lambda a, dt=torch.float32: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dt)
    dJ, dh0, dh1 = T(J), T(h0), T(h1)
    q0 = torch.empty(m * N0, dtype=torch.int8, device=dev)
    q1 = torch.empty(m * N1, dtype=torch.int8, device=dev)
    F0 = torch.empty(m * N0, dtype=torch.float32, device=dev)
    F1 = torch.empty(m * N1, dtype=torch.float32, device=dev)
    nbits = m * (N0 + N1) * (m if algo == "sa_naive" else 1)
    trace = torch.zeros((nbits + 31) // 32, dtype=torch.int32, device=dev)
    acc = torch.zeros(1, dtype=torch.int64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    seed = 99 + m
    assert L.sq103_randomize_spins(_p(q0), N0, m, ctypes.c_uint64(seed), ctypes.c_uint32(0), 0, sp) == 0
    assert L.sq103_randomize_spins(_p(q1), N1, m, ctypes.c_uint64(seed), ctypes.c_uint32(0), 1, sp) == 0
    torch.cuda.synchronize()
    a0, a1 = q0.cpu().numpy().reshape(m, N0), q1.cpu().numpy().reshape(m, N1)
    code = {"naive": orc.ALGO_NAIVE, "sa_naive": orc.ALGO_SA_NAIVE}[algo]
    for step, (G, beta) in enumerate([(3.0, 10.0), (0.5, 20.0), (0.05, 50.0)], start=1):
        trace.zero_()
        t = bench.BipartiteTask(J=dJ.data_ptr(), h0=dh0.data_ptr(), h1=dh1.data_ptr(), q0=q0.data_ptr(),
                                q1=q1.data_ptr(), F0=F0.data_ptr(), F1=F1.data_ptr(), trace=trace.data_ptr(),
                                accepted=acc.data_ptr(), G=None, beta=None, Gs=G, betas=beta, seed=seed, step0=step,
                                N0=N0, N1=N1, m=m, algo=code, nSteps=1, status=status.data_ptr())
        assert L.sq103_bipartite_anneal(ctypes.byref(t), sp) == 0
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        tr = trace.cpu().numpy().view(np.uint32)
        r0, r1, st = orc.bg_replay(h0, h1, J, m, code, seed, step, G, beta, a0, a1, tr, MARGIN_TOL)
        a0, a1 = q0.cpu().numpy().reshape(m, N0), q1.cpu().numpy().reshape(m, N1)
        assert np.array_equal(a0, r0) and np.array_equal(a1, r1)
        assert st["n_mismatch"] == st["n_mismatch_small"], st
