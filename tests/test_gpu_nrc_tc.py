"""tcgen05 (5th-generation tensor core) kernels of the radiance cache.

* the descriptor / instruction-descriptor / TMEM plumbing: one tcgen05.mma chain equals a PyTorch
  FP32 matmul of the same BF16 operands for every operand shape the MLP uses;
* the fused encode + 6-layer inference kernel equals the mma.sync twin on the same parameters
  (both BF16 x BF16 -> FP32; only the summation order differs), and no wait ran out.
"""
import ctypes as C

import pytest
import torch

from nrc_reference import random_features
from vierkant_gb300 import _lib
from vierkant_gb300.nrc import NeuralRadianceCache

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k,n", [(16, 16), (64, 64), (80, 64), (64, 16), (256, 32)])
def test_tc_gemm_matches_fp32_matmul(ctx, k, n):
    g = torch.Generator(device="cuda").manual_seed(k * 100 + n)
    a = torch.randn((128, k), device="cuda", generator=g).to(torch.bfloat16)
    b = torch.randn((n, k), device="cuda", generator=g).to(torch.bfloat16)
    d = torch.full((128, n), float("nan"), device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.check(_lib.lib().vkg_diag_tc_gemm(ctx.handle, C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), k, n,
                                           C.c_void_p(d.data_ptr()), C.c_void_p(err.data_ptr()),
                                           C.c_void_p(ctx.stream())), ctx.handle, "vkg_diag_tc_gemm")
    torch.cuda.synchronize()
    assert err.item() == 0
    ref = a.float() @ b.float().t()
    assert torch.isfinite(d).all()
    tol = 1e-5 * k * ref.abs().max().item()
    assert (d - ref).abs().max().item() <= tol, (d - ref).abs().max().item()


def _caches(ctx):
    caches = []
    for kind in (1, 2, 3):
        cfg = NeuralRadianceCache.default_config()
        cfg.log2_table_size = 16
        cfg.infer_kernel = kind
        caches.append(NeuralRadianceCache(ctx, cfg))
    i = caches[0].info()
    gen = torch.Generator(device="cuda").manual_seed(7)
    w = torch.randn(i.num_mlp_params, device="cuda", generator=gen) * 0.25
    grid = torch.randn(i.num_grid_params, device="cuda", generator=gen) * 0.5
    for c in caches:
        c.load_params(w, grid)
    return caches


def test_tc_inference_matches_mma_twin(ctx):
    mma, tcc, fused = _caches(ctx)
    assert [c.info().infer_kernel for c in (mma, tcc, fused)] == [1, 2, 3]
    for n in (1, 127, 128, 129, 70_001):
        feats = random_features(n, 100 + n)
        y1 = mma.infer(feats)
        for c in (tcc, fused):
            y2 = c.infer(feats)
            torch.cuda.synchronize()
            scale = y1.abs().mean().item()
            assert scale > 1e-3
            diff = (y1 - y2).abs()
            assert diff.mean().item() < 2e-3 * scale, (n, diff.mean().item(), scale)
            assert diff.max().item() < 5e-2 * max(scale, y1.abs().max().item() * 0.1), (n, diff.max().item())
    # the two tcgen05 kernels see identical BF16 inputs and issue identical MMAs
    y2, y3 = tcc.infer(feats), fused.infer(feats)
    assert torch.equal(y2, y3)
    assert tcc.info().kernel_error == 0 and fused.info().kernel_error == 0
    for c in (mma, tcc, fused):
        c.close()


def _grads(ctx, train_kernel, feats, targets, w, g):
    cfg = NeuralRadianceCache.default_config()
    cfg.log2_table_size = 16
    cfg.train_kernel = train_kernel
    c = NeuralRadianceCache(ctx, cfg)
    c.load_params(w, g)
    c.backward(feats, targets)
    torch.cuda.synchronize()
    i = c.info()
    from test_gpu_nrc import tensor_from
    out = (tensor_from(i.d_mlp_grads, i.num_mlp_params), tensor_from(i.d_grid_grads, i.num_grid_params), i)
    c.close()
    return out


@pytest.mark.parametrize("n", [1, 127, 4096, 70_001])
def test_tc_weight_gradients_match_fp32_kernel(ctx, n):
    """same BF16 activations and gradients, FP32 accumulation on both: equal up to summation order"""
    gen = torch.Generator(device="cuda").manual_seed(n)
    cfg = NeuralRadianceCache.default_config()
    cfg.log2_table_size = 16
    probe = NeuralRadianceCache(ctx, cfg)
    i = probe.info()
    w = torch.randn(i.num_mlp_params, device="cuda", generator=gen) * 0.2
    g = torch.randn(i.num_grid_params, device="cuda", generator=gen) * 0.5
    probe.close()
    feats = random_features(n, 40 + n)
    targets = torch.rand((n, 3), device="cuda", generator=gen)
    w1, g1, i1 = _grads(ctx, 1, feats, targets, w, g)
    w2, g2, i2 = _grads(ctx, 2, feats, targets, w, g)
    assert i1.train_kernel == 1 and i2.train_kernel == 2 and i2.kernel_error == 0
    # the hash-grid gradients do not depend on the weight-gradient kernel (float atomics: order only)
    assert (g1 - g2).abs().max().item() <= 1e-5 * g1.abs().max().item() + 1e-9
    scale = w1.abs().max().item()
    assert scale > 0
    assert (w1 - w2).abs().max().item() <= 1e-4 * scale + 1e-7, (w1 - w2).abs().max().item()


def test_tc_training_fits_like_fp32(ctx):
    from test_gpu_nrc import _field
    test = random_features(8192, 999)
    tt = _field(test)
    errs = []
    for kind in (1, 2):
        cfg = NeuralRadianceCache.default_config()
        cfg.train_kernel = kind
        c = NeuralRadianceCache(ctx, cfg)
        for step in range(200):
            feats = random_features(65536, 1000 + step)
            c.train_step(feats, _field(feats))
        errs.append(((c.infer(test) - tt).abs().mean() / tt.abs().mean()).item())
        assert c.info().kernel_error == 0
        c.close()
    print("held-out relative error fp32 / tcgen05 weight gradients:", errs)
    assert errs[1] < 0.18 and abs(errs[1] - errs[0]) < 0.06


def _wait_probe(ctx, num_ctas, limit_ns):
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    elapsed = torch.zeros(1, dtype=torch.int64, device="cuda")
    _lib.check(_lib.lib().vkg_diag_wait_timeout(ctx.handle, num_ctas, limit_ns, C.c_void_p(err.data_ptr()),
                                                C.c_void_p(elapsed.data_ptr()), C.c_void_p(ctx.stream())),
               ctx.handle, "vkg_diag_wait_timeout")
    torch.cuda.synchronize()
    return err.item(), elapsed.item()


def test_bounded_wait_runs_out_and_returns(ctx):
    """A wait that nothing ends gives up after its limit: the kernel sets the error bit, takes the
    second bounded wait of the error path, frees its TMEM and returns; the context stays usable and
    the tcgen05 kernels that follow allocate TMEM and run normally."""
    limit = 2_000_000  # 2 ms instead of the kernels' 1 s
    for num_ctas in (1, 2 * 152):
        err, elapsed = _wait_probe(ctx, num_ctas, limit)
        assert err == 1
        # both waits of a CTA ran to their limit, and no CTA hung beyond it
        assert 2 * limit <= elapsed < 50 * limit, elapsed
    # TMEM was freed: tcgen05 kernels after the probe still allocate, multiply and finish in time
    test_tc_gemm_matches_fp32_matmul(ctx, 64, 64)
    cache = NeuralRadianceCache(ctx, NeuralRadianceCache.default_config())
    x = random_features(4096, seed=3)
    cache.infer(x)
    torch.cuda.synchronize()
    assert cache.info().kernel_error == 0
    cache.close()


def test_tc_training_forward_backward_match_mma(ctx):
    """train_kernel 3 runs the training forward and the backward through the layers on the pipelined
    tcgen05 kernels: the gradients equal train_kernel 2's (mma.sync) up to the BF16 rounding of
    activations and layer gradients whose FP32 sums differ in summation order"""
    n = 20_000
    gen = torch.Generator(device="cuda").manual_seed(5)
    cfg = NeuralRadianceCache.default_config()
    cfg.log2_table_size = 16
    probe = NeuralRadianceCache(ctx, cfg)
    i = probe.info()
    w = torch.randn(i.num_mlp_params, device="cuda", generator=gen) * 0.2
    g = torch.randn(i.num_grid_params, device="cuda", generator=gen) * 0.5
    probe.close()
    feats = random_features(n, 77)
    targets = torch.rand((n, 3), device="cuda", generator=gen)
    w2, g2, i2 = _grads(ctx, 2, feats, targets, w, g)
    w3, g3, i3 = _grads(ctx, 3, feats, targets, w, g)
    assert i2.train_kernel == 2 and i3.train_kernel == 3 and i3.kernel_error == 0
    cos = lambda a, b: float((a * b).sum() / (a.norm() * b.norm()))
    assert cos(w2, w3) > 0.9999 and cos(g2, g3) > 0.9999, (cos(w2, w3), cos(g2, g3))
    assert (w2 - w3).abs().max().item() <= 2e-2 * w2.abs().max().item()
