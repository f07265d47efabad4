"""tcgen05 field refresh (TMA-fed, TMEM-accumulated, exact digit contraction)
against the FP64 oracle and the SIMT spin GEMM, through the kernel layer of the
C ABI; plus its bounded waits giving up on purpose and the device staying
usable."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SKIP_FIRST_COPY, SHORT_WAITS = 1, 2


def _lib():
    torch = pytest.importorskip("torch")
    from sqaod_gb300 import _lib as L_
    L = L_.lib()
    L.sq103_tc_digits_bytes.restype = ctypes.c_ulonglong
    L.sq103_tc_spins_bytes.restype = ctypes.c_ulonglong
    return torch, L


def _refresh(torch, L, B, q, R, K, transpose=0, flags=0):
    """F = q . B^T (q: m x K spins) with B = J (R x K) or J^T (J: K x R when transposed)."""
    dev = q.device
    m = q.shape[0]
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    D = torch.empty(int(L.sq103_tc_digits_bytes(R, K)), dtype=torch.uint8, device=dev)
    A = torch.empty(int(L.sq103_tc_spins_bytes(m, K)), dtype=torch.uint8, device=dev)
    F = torch.full((m, R), float("nan"), dtype=torch.float32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    assert L.sq103_tc_make_digits(P(B), B.shape[1], R, K, transpose, P(D), stream) == 0
    assert L.sq103_tc_refresh(P(D), R, K, P(q), K, m, P(A), P(F), R, flags, P(status), stream) == 0
    torch.cuda.synchronize()
    return F, int(status.item())


@pytest.mark.parametrize("N,m", [(256, 16), (512, 64), (1024, 256), (4096, 256), (200, 7), (384, 130), (64, 1)])
def test_tc_field_refresh_dense(N, m):
    torch, L = _lib()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(N + m)
    W = rng.uniform(-1, 1, (N, N))
    W = (np.triu(W) + np.triu(W, 1).T).astype(np.float32)
    J = torch.from_numpy((-0.25 * W) * (1 - np.eye(N, dtype=np.float32))).to(dev).contiguous()
    q = torch.from_numpy(rng.choice(np.array([-1, 1], np.int8), (m, N))).to(dev).contiguous()
    F_tc, st = _refresh(torch, L, J, q, N, N)
    assert st == 0
    F_simt = torch.empty((m, N), dtype=torch.float32, device=dev)
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    assert L.sq103_dense_field_refresh(P(J), N, P(q), P(F_simt), N, m,
                                       ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
    torch.cuda.synchronize()
    F64 = q.double() @ J.double()  # F[y][i] = sum_j q[y][j] J[j][i] = sum_j J[i][j] q[y][j]
    scale = float(F64.abs().max()) + 1.0
    err_tc = float((F_tc.double() - F64).abs().max())
    err_simt = float((F_simt.double() - F64).abs().max())
    assert not torch.isnan(F_tc).any()
    print("N=%d m=%d  max |F - F64| / (max|F64| + 1): tcgen05 %.2e  simt %.2e" % (N, m, err_tc / scale,
                                                                                  err_simt / scale))
    # exact digit contraction: only the 31-bit quantisation of J and the final fp32 rounding remain
    assert err_tc <= 2e-7 * scale, (err_tc, err_simt, scale)
    # and at most the fp32 rounding of the result plus the quantisation: within a few ulps of F64
    ulp = torch.finfo(torch.float32).eps * F64.abs().clamp_min(1e-30)
    assert bool(((F_tc.double() - F64).abs() <= ulp + 4e-9 * scale).all())


@pytest.mark.parametrize("N0,N1,m", [(1024, 1024, 64), (40, 200, 6), (333, 1000, 5)])
def test_tc_field_refresh_bipartite(N0, N1, m):
    """The bipartite half-step fields: F1 = q0 J^T (rows of J) and F0 = q1 J
    (columns: the transposed digits)."""
    torch, L = _lib()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(N0 + N1 + m)
    J = torch.from_numpy((-0.25 * rng.uniform(-1, 1, (N1, N0))).astype(np.float32)).to(dev).contiguous()
    q0 = torch.from_numpy(rng.choice(np.array([-1, 1], np.int8), (m, N0))).to(dev).contiguous()
    q1 = torch.from_numpy(rng.choice(np.array([-1, 1], np.int8), (m, N1))).to(dev).contiguous()
    F1, st1 = _refresh(torch, L, J, q0, N1, N0)
    F0, st0 = _refresh(torch, L, J, q1, N0, N1, transpose=1)
    assert st0 == 0 and st1 == 0
    for F, ref in ((F1, q0.double() @ J.double().T), (F0, q1.double() @ J.double())):
        scale = float(ref.abs().max()) + 1.0
        assert float((F.double() - ref).abs().max()) <= 2e-7 * scale


def test_tc_wait_gives_up_and_device_stays_usable():
    """The producer withholds the first K block's copies and waits give up
    after 1 ms: the kernel returns status 1 instead of hanging; the next
    refresh on the same device is exact again."""
    torch, L = _lib()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(3)
    N, m = 512, 32
    J = torch.from_numpy(rng.uniform(-0.25, 0.25, (N, N)).astype(np.float32)).to(dev).contiguous()
    q = torch.from_numpy(rng.choice(np.array([-1, 1], np.int8), (m, N))).to(dev).contiguous()
    _, st = _refresh(torch, L, J, q, N, N, flags=SKIP_FIRST_COPY | SHORT_WAITS)
    assert st == 1
    F, st = _refresh(torch, L, J, q, N, N)
    assert st == 0
    ref = q.double() @ J.double().T
    assert float((F.double() - ref).abs().max()) <= 2e-7 * (float(ref.abs().max()) + 1.0)


def test_tc_rejects_bad_arguments():
    torch, L = _lib()
    assert L.sq103_tc_make_digits(None, 64, 64, 64, 0, None, None) != 0
    assert L.sq103_tc_refresh(None, 64, 64, None, 64, 8, None, None, 64, 0, None, None) != 0
