"""The tcgen05 BF16 GEMM against a plain PyTorch FP32 reference of the same
op (bf16 operands, fp32 accumulation)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16_bits(x):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(x, np.float32)).to(torch.bfloat16)
    return t.view(torch.int16).numpy().view(np.uint16), t.to(torch.float32)


@pytest.mark.parametrize("M,N,K,act", [(128, 128, 64, 0), (256, 256, 256, 0), (384, 128, 128, 1),
                                       (200, 72, 64, 1), (1024, 256, 256, 1), (256, 200, 512, 1),
                                       (130, 300, 192, 0), (512, 128, 1024, 0)])
def test_tc_gemm_matches_torch_fp32(M, N, K, act):
    torch = pytest.importorskip("torch")
    import pticm
    rng = np.random.default_rng(M + N + K)
    a_bits, a = _bf16_bits(rng.standard_normal((M, K)))
    b_bits, b = _bf16_bits(rng.standard_normal((N, K)) / np.sqrt(K))
    bias = rng.standard_normal(N).astype(np.float32)
    out = np.zeros((M, N), np.float32)
    out_bf16 = np.zeros((M, N), np.uint16)
    L = pticm.lib()
    L.pticm_tc_gemm_check.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                      C.c_void_p, C.c_void_p]
    rc = L.pticm_tc_gemm_check(M, N, K, a_bits.ctypes.data, b_bits.ctypes.data, bias.ctypes.data, act,
                               out.ctypes.data, out_bf16.ctypes.data)
    assert rc == 0, L.pticm_last_error()
    pre = a @ b.T + torch.from_numpy(bias)
    # the FP32 output is the pre-activation sum
    assert np.allclose(out, pre.numpy(), rtol=1e-4, atol=1e-3), np.abs(out - pre.numpy()).max()
    # the BF16 output is the activation of it, rounded to BF16 (one BF16 ulp
    # of the value plus the fast exponential's error)
    post = torch.nn.functional.silu(pre) if act == 1 else pre
    got = torch.from_numpy(out_bf16.view(np.int16)).view(torch.bfloat16).to(torch.float32).numpy()
    want = post.numpy()
    assert np.all(np.abs(got - want) <= 2.0 ** -7 * np.abs(want) + 1e-3), np.abs(got - want).max()


def test_tc_gemm_bench_runs():
    import ctypes as C
    import pticm
    L = pticm.lib()
    L.pticm_tc_gemm_bench.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    ms, tf = C.c_double(), C.c_double()
    assert L.pticm_tc_gemm_bench(4096, 256, 256, 5, C.byref(ms), C.byref(tf)) == 0
    assert ms.value > 0 and tf.value > 0
