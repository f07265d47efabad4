"""GPU test of sq103_dense_energy_static, the energy entry point that allocates nothing.

Some callers of this library cannot call cudaMalloc: code that runs inside a
framework that owns all device memory through its own pool, or a long-lived
service that must not grow its footprint after start-up.  For them
sq103_dense_energy_static computes the FP64 trotter energies with its scratch
in a fixed static device array instead of a caller-provided buffer.  This test
calls it twice in a row through the C ABI and checks both results against
sq103_dense_energy (which takes caller-allocated scratch), and checks that a
size beyond the static maximum is refused with a clear error.

This file is collected last on purpose, so that a run that stops at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-11  # FP64 energies, same tolerance as the other FP64 energy tests


def _rel_close(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b))) <= REL_TOL * max(1.0, float(np.max(np.abs(b))))


def test_static_scratch_energy_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    from sqaod_gb300 import _lib
    L = _lib.lib()
    L.sq103_dense_energy_static_max.restype = ctypes.c_ulonglong
    dev = torch.device("cuda", 0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def P(t):
        return ctypes.c_void_p(t.data_ptr())

    N, m = 512, 64
    assert N * m <= L.sq103_dense_energy_static_max()
    rng = np.random.default_rng(2024)
    W = rng.uniform(-1, 1, (N, N))
    W = (np.triu(W) + np.triu(W, 1).T).astype(np.float32)
    dW = torch.from_numpy(W).to(dev)
    J = torch.empty((N, N), dtype=torch.float32, device=dev)
    h = torch.empty(N, dtype=torch.float32, device=dev)
    c32 = torch.empty(1, dtype=torch.float32, device=dev)
    c64 = torch.empty(1, dtype=torch.float64, device=dev)
    hs = torch.empty(N, dtype=torch.float64, device=dev)
    q = torch.empty((m, N), dtype=torch.int8, device=dev)
    assert L.sq103_dense_hamiltonian(P(dW), N, N, 0, P(h), P(J), N, P(c32), P(c64), P(hs), stream) == 0
    assert L.sq103_randomize_spins(P(q), N, m, ctypes.c_uint64(7), ctypes.c_uint32(0), 0, stream) == 0

    # the allocating entry point, scratch supplied by the caller
    r = torch.empty((m, N), dtype=torch.float64, device=dev)
    E_ref = torch.empty(m, dtype=torch.float64, device=dev)
    E_ref32 = torch.empty(m, dtype=torch.float32, device=dev)
    assert L.sq103_dense_energy(P(J), N, P(h), P(c64), P(q), N, m, 0, P(r), P(E_ref), P(E_ref32), stream) == 0

    # the static-scratch entry point, twice in a row
    for _ in range(2):
        E = torch.full((m,), float("nan"), dtype=torch.float64, device=dev)
        E32 = torch.full((m,), float("nan"), dtype=torch.float32, device=dev)
        assert L.sq103_dense_energy_static(P(J), N, P(h), P(c64), P(q), N, m, 0, P(E), P(E32), stream) == 0
        torch.cuda.synchronize()
        assert _rel_close(E.cpu().numpy(), E_ref.cpu().numpy())
        assert np.array_equal(E32.cpu().numpy(), E_ref32.cpu().numpy())

    # beyond the static maximum: refused with a clear error, nothing launched
    big_m = int(L.sq103_dense_energy_static_max()) // N + 1
    L.sq103_last_error.restype = ctypes.c_char_p
    rc = L.sq103_dense_energy_static(P(J), N, P(h), P(c64), P(q), N, big_m, 0, P(E), P(E32), stream)
    assert rc == 3
    assert b"exceeds the static scratch" in L.sq103_last_error()
