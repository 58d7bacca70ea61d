"""The tensor-core (tcgen05 + TMEM) kernels of the learned constitutive surrogate against plain
references: the BF16 GEMM they are built on against an FP64 product of the same BF16 inputs."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    """float32 -> bfloat16 bit patterns, round to nearest even."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def bf16_value(b):
    return (np.asarray(b, np.uint16).astype(np.uint32) << 16).view(np.float32)


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.parametrize("M,N,K", [(128, 16, 16), (256, 64, 64), (200, 64, 128), (128, 256, 256), (384, 16, 64)])
def test_tc_gemm_matches_fp64(gpu_lib, torch_cuda, M, N, K):
    """C = A B^T on the tensor cores (BF16 operands, FP32 accumulation in TMEM) equals the FP64
    product of the same BF16 values to FP32 accumulation error, for full and partial 128-row
    tiles, N from 16 to 256 and K from 16 to 256."""
    torch = torch_cuda
    from graphyt_gb300 import _lib
    rng = np.random.default_rng(M * 1000 + N + K)
    a = bf16_bits(rng.standard_normal((M, K)))
    b = bf16_bits(rng.standard_normal((N, K)))
    A = torch.from_numpy(a.view(np.int16)).cuda()
    B = torch.from_numpy(b.view(np.int16)).cuda()
    C = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    rc = gpu_lib.gy_tc_gemm_bf16(ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()),
                                 ctypes.c_void_p(C.data_ptr()), M, N, K, ctypes.c_void_p(status.data_ptr()),
                                 ctypes.c_void_p(stream.cuda_stream))
    assert rc == _lib.GY_OK
    stream.synchronize()
    assert int(status.item()) == 0
    af, bf = bf16_value(a).astype(np.float64), bf16_value(b).astype(np.float64)
    want = af @ bf.T
    scale = np.abs(af) @ np.abs(bf).T
    got = C.cpu().numpy().astype(np.float64)
    assert np.all(np.abs(got - want) <= 1e-5 * scale + 1e-30)


def test_tc_gemm_rejects_bad_shapes(gpu_lib):
    from graphyt_gb300 import _lib
    p = ctypes.c_void_p(16)
    for M, N, K in [(0, 16, 16), (128, 8, 16), (128, 24, 16), (128, 512, 16), (128, 16, 8), (128, 16, 512)]:
        assert gpu_lib.gy_tc_gemm_bf16(p, p, p, M, N, K, None, None) == _lib.GY_ERR_ARG


def mlp_params(rng, in_mean, in_std, out_mean, out_std):
    """A packed parameter vector in the library's layout, weights ~ N(0, 1/fan_in)."""
    W1 = rng.standard_normal((16, 64)) / 4.0
    W2 = rng.standard_normal((64, 64)) / 8.0
    W3 = rng.standard_normal((64, 7)) / 8.0
    b1, b2, b3 = 0.1 * rng.standard_normal(64), 0.1 * rng.standard_normal(64), 0.1 * rng.standard_normal(7)
    return np.concatenate([W1.ravel(), b1, W2.ravel(), b2, W3.ravel(), b3, in_mean, in_std, out_mean,
                           out_std]).astype(np.float32), (W1, b1, W2, b2, W3, b3)


def mlp_reference(x, prm, bf16_like):
    """FP32/FP64 reference of the surrogate MLP; bf16_like rounds the operands the tensor
    cores see (normalised inputs, weights, hidden activations) to BF16."""
    o = 0
    def take(k):
        nonlocal o
        v = prm[o:o + k].astype(np.float64)
        o += k
        return v
    W1, b1 = take(16 * 64).reshape(16, 64), take(64)
    W2, b2 = take(64 * 64).reshape(64, 64), take(64)
    W3, b3 = take(64 * 7).reshape(64, 7), take(7)
    im, isd, om, osd = take(16), take(16), take(7), take(7)
    r = (lambda a: bf16_value(bf16_bits(a)).astype(np.float64)) if bf16_like else (lambda a: a)
    silu = lambda z: z / (1.0 + np.exp(-z))
    xn = r(((x - im) / isd).astype(np.float32))
    h1 = r(silu(xn @ r(W1) + b1).astype(np.float32))
    h2 = r(silu(h1 @ r(W2) + b2).astype(np.float32))
    return (h2 @ r(W3) + b3) * osd + om


def test_mlp_forward_matches_reference(gpu_lib, torch_cuda):
    """The surrogate MLP's forward pass on the tensor cores (BF16 operands, FP32 accumulation)
    against a reference with the same BF16 roundings (relative L2 <= 2e-3, the width of one
    BF16 rounding flip) and against the plain FP32 MLP (<= 3e-2: the BF16 roundings
    themselves), over partial and full 128-row tiles."""
    torch = torch_cuda
    from graphyt_gb300 import _lib
    assert gpu_lib.gy_mlp_param_count() == 16 * 64 + 64 + 64 * 64 + 64 + 64 * 7 + 7 + 16 + 16 + 7 + 7
    rng = np.random.default_rng(3)
    in_mean, in_std = rng.standard_normal(16), 0.5 + rng.random(16)
    out_mean, out_std = rng.standard_normal(7), 0.5 + rng.random(7)
    prm, _ = mlp_params(rng, in_mean, in_std, out_mean, out_std)
    for n in (1, 127, 128, 1000, 40_000):
        x = (in_mean + in_std * rng.standard_normal((n, 16))).astype(np.float32)
        P = torch.from_numpy(prm).cuda()
        X = torch.from_numpy(x).cuda()
        Y = torch.full((n, 7), float("nan"), dtype=torch.float32, device="cuda")
        status = torch.zeros(1, dtype=torch.int32, device="cuda")
        stream = torch.cuda.current_stream()
        rc = gpu_lib.gy_mlp_forward(ctypes.c_void_p(P.data_ptr()), ctypes.c_void_p(X.data_ptr()), n,
                                    ctypes.c_void_p(Y.data_ptr()), ctypes.c_void_p(status.data_ptr()),
                                    ctypes.c_void_p(stream.cuda_stream))
        assert rc == _lib.GY_OK
        stream.synchronize()
        assert int(status.item()) == 0
        got = Y.cpu().numpy().astype(np.float64)
        like = mlp_reference(x.astype(np.float64), prm, True)
        fp32 = mlp_reference(x.astype(np.float64), prm, False)
        def rel(a, b):
            return np.linalg.norm(a - b) / np.linalg.norm(b)
        assert rel(got, like) <= 2e-3, (n, rel(got, like))
        assert rel(got, fp32) <= 3e-2, (n, rel(got, fp32))
