"""tcgen05 field refresh (TMA-fed, TMEM-accumulated) against the FP64 oracle and
the SIMT spin GEMM, through the kernel layer of the C ABI."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(N, m, seed):
    torch = pytest.importorskip("torch")
    from sqaod_gb300 import _lib
    L = _lib.lib()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(seed)
    W = rng.uniform(-1, 1, (N, N))
    W = (np.triu(W) + np.triu(W, 1).T).astype(np.float32)
    J = torch.from_numpy((-0.25 * W) * (1 - np.eye(N, dtype=np.float32))).to(dev).contiguous()
    q = torch.from_numpy(rng.choice(np.array([-1, 1], np.int8), (m, N))).to(dev).contiguous()
    return torch, L, dev, J, q


@pytest.mark.parametrize("N,m", [(256, 16), (512, 64), (1024, 256), (4096, 256), (200, 7), (384, 130)])
def test_tc_field_refresh(N, m):
    torch, L, dev, J, q = _setup(N, m, N + m)
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    Kp = L.sq103_tc_kpad(N)
    B = torch.empty((N, Kp), dtype=torch.bfloat16, device=dev)
    A = torch.empty((m, Kp), dtype=torch.bfloat16, device=dev)
    F_tc = torch.full((m, N), float("nan"), dtype=torch.float32, device=dev)
    F_simt = torch.empty((m, N), dtype=torch.float32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    assert L.sq103_tc_split_couplings(P(J), N, N, P(B), stream) == 0
    # the three bf16 parts represent J exactly
    parts = B[:, :3 * N].float().reshape(N, 3, N).sum(1)
    assert torch.equal(parts, J)
    assert L.sq103_tc_field_refresh(P(B), P(q), P(A), P(F_tc), N, m, P(status), stream) == 0
    assert L.sq103_dense_field_refresh(P(J), N, P(q), P(F_simt), N, m, stream) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    F64 = q.double() @ J.double()  # F[y][i] = sum_j q[y][j] J[j][i] = sum_j J[i][j] q[y][j]
    scale = float(F64.abs().max()) + 1.0
    err_tc = float((F_tc.double() - F64).abs().max())
    err_simt = float((F_simt.double() - F64).abs().max())
    assert not torch.isnan(F_tc).any()
    print("N=%d m=%d  max |F - F64| / max|F64|: tcgen05 %.2e  simt %.2e" % (N, m, err_tc / scale, err_simt / scale))
    # exact products, tensor-core fp32 accumulation over K = 3N: measured
    # 1.6e-6 (N=256) to 1.1e-5 (N=4096) of the row scale
    assert err_tc <= 2e-5 * scale, (err_tc, err_simt, scale)
    # the SIMT GEMM (sequential fp32 FMAs over 32-wide chunks, FP64 across chunks)
    assert err_simt <= 1e-6 * scale, (err_tc, err_simt, scale)
