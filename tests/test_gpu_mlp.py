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


def test_lost_arrival_ends_in_a_status(gpu_lib, torch_cuda):
    """A tensor-core wait whose arrival never comes gives up: a block waiting on an mbarrier that
    nothing completes ends within a second with the timeout bit set, and the context stays
    usable (a GEMM afterwards is exact)."""
    torch = torch_cuda
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    elapsed = torch.zeros(1, dtype=torch.int64, device="cuda")
    assert gpu_lib.gy_tc_wait_check(ctypes.c_void_p(status.data_ptr()), ctypes.c_void_p(elapsed.data_ptr()), None) == 0
    torch.cuda.synchronize()
    assert status.item() & 4
    assert 1e6 < elapsed.item() < 2e9, elapsed.item()  # gave up after a fraction of a second
    a = bf16_bits(np.ones((128, 16), np.float32))
    A = torch.from_numpy(a.view(np.int16)).cuda()
    Cm = torch.zeros((128, 16), dtype=torch.float32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert gpu_lib.gy_tc_gemm_bf16(ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(A.data_ptr()),
                                   ctypes.c_void_p(Cm.data_ptr()), 128, 16, 16, ctypes.c_void_p(st.data_ptr()),
                                   None) == 0
    torch.cuda.synchronize()
    assert st.item() == 0 and torch.all(Cm == 16.0)


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


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_mlp_gradient_matches_autograd(gpu_lib, torch_cuda):
    """One pass of the training kernel (tensor-core forward, backward and weight gradients,
    BF16 operands) against FP32 autograd of the same MLP and loss: the gradient of every
    parameter block within 5e-2 (relative L2; BF16 activations and gradient tiles), the loss
    within 1e-2."""
    torch = torch_cuda
    from graphyt_gb300 import _lib
    rng = np.random.default_rng(5)
    in_mean, in_std = rng.standard_normal(16), 0.5 + rng.random(16)
    out_mean, out_std = rng.standard_normal(7), 0.5 + rng.random(7)
    prm, _ = mlp_params(rng, in_mean, in_std, out_mean, out_std)
    n = 512
    x = (in_mean + in_std * rng.standard_normal((n, 16))).astype(np.float32)
    t = (out_mean + out_std * rng.standard_normal((n, 7))).astype(np.float32)
    P, X, T = (torch.from_numpy(a).cuda() for a in (prm, x, t))
    G = torch.zeros(len(prm), dtype=torch.float32, device="cuda")
    Lo = torch.zeros(1, dtype=torch.float32, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    assert gpu_lib.gy_mlp_grad(_ptr(P), _ptr(X), _ptr(T), n, _ptr(G), _ptr(Lo), _ptr(st),
                               ctypes.c_void_p(stream.cuda_stream)) == _lib.GY_OK
    stream.synchronize()
    assert int(st.item()) == 0
    # FP32 autograd reference
    p = torch.from_numpy(prm.astype(np.float64)).requires_grad_(True)
    o = 0
    def take(k, shape):
        nonlocal o
        v = p[o:o + k].reshape(shape)
        o += k
        return v
    W1, b1 = take(1024, (16, 64)), take(64, (64,))
    W2, b2 = take(4096, (64, 64)), take(64, (64,))
    W3, b3 = take(448, (64, 7)), take(7, (7,))
    im, isd = torch.from_numpy(in_mean), torch.from_numpy(in_std)
    om, osd = torch.from_numpy(out_mean), torch.from_numpy(out_std)
    xn = (torch.from_numpy(x.astype(np.float64)) - im) / isd
    tn = (torch.from_numpy(t.astype(np.float64)) - om) / osd
    h1 = torch.nn.functional.silu(xn @ W1 + b1)
    h2 = torch.nn.functional.silu(h1 @ W2 + b2)
    y = h2 @ W3 + b3
    loss = ((y - tn) ** 2).mean()
    loss.backward()
    want = p.grad.numpy()
    got = G.cpu().numpy().astype(np.float64)
    blocks = {"W1": (0, 1024), "b1": (1024, 1088), "W2": (1088, 5184), "b2": (5184, 5248), "W3": (5248, 5696),
              "b3": (5696, 5703)}
    for name, (a, b) in blocks.items():
        err = np.linalg.norm(got[a:b] - want[a:b]) / np.linalg.norm(want[a:b])
        assert err <= 5e-2, (name, err)
    assert np.all(got[5703:] == 0.0)  # the normalisation is not trained
    lv = float(loss.detach())
    assert abs(float(Lo.item()) - lv) <= 1e-2 * lv


def test_mlp_training_fits_a_smooth_map(gpu_lib, torch_cuda):
    """gy_mlp_train (tensor-core training steps replayed from a CUDA graph, Adam) fits a smooth
    16 -> 7 map: the normalised loss falls below 2 % of its initial value, and the trained
    forward pass reproduces held-out targets to a relative L2 of 0.15."""
    torch = torch_cuda
    from graphyt_gb300 import _lib
    rng = np.random.default_rng(9)
    n = 1 << 16
    A = rng.standard_normal((16, 7)) / 4.0
    def f(x):
        return np.tanh(x @ A) + 0.3 * np.sin(x[:, :7])
    x = rng.standard_normal((n, 16)).astype(np.float32)
    t = f(x.astype(np.float64)).astype(np.float32)
    P = torch.zeros(gpu_lib.gy_mlp_param_count(), dtype=torch.float32, device="cuda")
    X, T = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    s = ctypes.c_void_p(stream.cuda_stream)
    l0, l1 = ctypes.c_float(), ctypes.c_float()
    assert gpu_lib.gy_mlp_train(_ptr(P), _ptr(X), _ptr(T), n, 1, 4096, ctypes.c_float(1e-3), 1, 1,
                                ctypes.byref(l0), _ptr(st), s) == _lib.GY_OK
    assert gpu_lib.gy_mlp_train(_ptr(P), _ptr(X), _ptr(T), n, 3000, 4096, ctypes.c_float(2e-3), 1, 0,
                                ctypes.byref(l1), _ptr(st), s) == _lib.GY_OK
    stream.synchronize()
    assert int(st.item()) == 0
    assert l1.value < 0.02 * l0.value, (l0.value, l1.value)
    xv = rng.standard_normal((4096, 16)).astype(np.float32)
    Y = torch.empty((4096, 7), dtype=torch.float32, device="cuda")
    assert gpu_lib.gy_mlp_forward(_ptr(P), _ptr(torch.from_numpy(xv).cuda()), 4096, _ptr(Y), _ptr(st), s) == _lib.GY_OK
    stream.synchronize()
    want = f(xv.astype(np.float64))
    err = np.linalg.norm(Y.cpu().numpy() - want) / np.linalg.norm(want)
    assert err <= 0.15, err
