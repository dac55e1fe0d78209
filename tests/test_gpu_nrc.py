"""Neural radiance cache kernels against the PyTorch reference (tests/nrc_reference.py):
forward predictions, loss gradients of every MLP weight and of the hash grid, Adam, and training."""
import ctypes as C

import numpy as np
import pytest
import torch

from nrc_reference import (encode, forward, random_features, relative_l2, split_weights)
from vierkant_gb300.nrc import NeuralRadianceCache

pytestmark = pytest.mark.gpu


def tensor_from(ptr, n, dtype=torch.float32):
    out = torch.empty(n, dtype=dtype, device="cuda")
    import glob
    for cand in ["libcudart.so.13", "libcudart.so"] + sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*")):
        try:
            rt = C.CDLL(cand)
            break
        except OSError:
            continue
    rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    assert rt.cudaMemcpy(C.c_void_p(out.data_ptr()), C.c_void_p(ptr), C.c_size_t(out.numel() * out.element_size()), 3) == 0
    return out


@pytest.fixture(params=[2, 3], ids=["mma_fwd_bwd", "tcgen05_fwd_bwd"])
def cache(ctx, request):
    cfg = NeuralRadianceCache.default_config()
    cfg.log2_table_size = 14  # small tables keep the FP64 reference quick
    cfg.train_kernel = request.param  # forward / backward on mma.sync (2) or tcgen05 (3)
    c = NeuralRadianceCache(ctx, cfg)
    yield c
    c.close()


def reference_inputs(c: NeuralRadianceCache):
    i = c.info()
    res = [i.level_resolution[l] for l in range(i.levels)]
    w = tensor_from(i.d_mlp_params, i.num_mlp_params)
    g = tensor_from(i.d_grid_params, i.num_grid_params)
    return res, i.table_size, w, g


def test_level_resolutions_and_init(cache):
    from nrc_reference import level_resolutions
    i = cache.info()
    assert [i.level_resolution[l] for l in range(16)] == level_resolutions()
    _, _, w, g = reference_inputs(cache)
    assert g.abs().max().item() <= 1e-4 and w.abs().max().item() < 0.5
    ws = split_weights(w)
    assert torch.all(ws[-1][:, 3:] == 0)


def test_forward_matches_reference(cache):
    feats = random_features(8192, 1)
    # non-trivial grid values so the encoding matters
    res, table, w, g = reference_inputs(cache)
    g = torch.randn(g.shape, device="cuda") * 0.5
    w = w * 3.0
    cache.load_params(w, g)
    y = cache.infer(feats)
    X = encode(feats, g, res, table, (-1, -1, -1), (1, 1, 1))
    ref = forward(X, split_weights(w))
    err = (y - ref).abs()
    scale = ref.abs().mean().item()
    assert scale > 1e-2
    assert err.max().item() < 0.05 * max(scale, ref.abs().max().item() * 0.1), (err.max().item(), scale)
    assert err.mean().item() < 0.01 * scale


def test_gradients_match_reference(cache):
    feats = random_features(4096, 2)
    res, table, w, g = reference_inputs(cache)
    g = torch.randn(g.shape, device="cuda") * 0.5
    w = w * 3.0
    cache.load_params(w, g)
    targets = torch.rand((4096, 3), device="cuda") * 2
    cache.backward(feats, targets)
    torch.cuda.synchronize()
    i = cache.info()
    gw = tensor_from(i.d_mlp_grads, i.num_mlp_params)
    gg = tensor_from(i.d_grid_grads, i.num_grid_params)
    # FP64 reference on the same BF16-rounded weights / activations (rounding treated as identity)
    w64 = w.double().clone().requires_grad_(True)
    g64 = g.double().clone().requires_grad_(True)
    X = encode(feats, g64, res, table, (-1, -1, -1), (1, 1, 1))
    y = forward(X, split_weights(w64))
    loss = relative_l2(y, targets.double())
    loss.backward()
    for name, a, b in (("mlp", gw.double(), w64.grad), ("grid", gg.double(), g64.grad)):
        cos = torch.nn.functional.cosine_similarity(a, b, dim=0).item()
        rel = ((a - b).norm() / b.norm()).item()
        print(name, "cosine", cos, "relative error", rel)
        assert cos > 0.995 and rel < 0.08, (name, cos, rel)
    # per layer as well
    for l, (a, b) in enumerate(zip(split_weights(gw.double()), split_weights(w64.grad))):
        if b.norm() > 0:
            assert torch.nn.functional.cosine_similarity(a.flatten(), b.flatten(), dim=0).item() > 0.99, l


def test_adam_step_matches_formula(cache):
    feats = random_features(2048, 3)
    targets = torch.rand((2048, 3), device="cuda")
    _, _, w0, _ = reference_inputs(cache)
    cache.backward(feats, targets)
    torch.cuda.synchronize()
    i = cache.info()
    gw = tensor_from(i.d_mlp_grads, i.num_mlp_params)
    cache.adam_step()
    torch.cuda.synchronize()
    _, _, w1, _ = reference_inputs(cache)
    cfg = cache.config
    m = (1 - cfg.beta1) * gw
    v = (1 - cfg.beta2) * gw * gw
    expect = w0 - cfg.learning_rate * (m / (1 - cfg.beta1)) / (torch.sqrt(v / (1 - cfg.beta2)) + cfg.epsilon)
    assert torch.allclose(w1, expect, rtol=1e-5, atol=1e-7)
    assert cache.info().step == 1
    # gradients were consumed
    assert tensor_from(cache.info().d_mlp_grads, i.num_mlp_params).abs().max().item() == 0.0


def _field(f):
    p = f[:, 0:3]
    return torch.stack([1 + torch.sin(3 * p[:, 0]), 1 + 0.5 * torch.cos(2 * p[:, 1]) * p[:, 2], f[:, 10] * 2],
                       dim=1) * (1 + f[:, 6:7].clamp(min=0))


def test_training_fits_a_smooth_radiance_field(ctx):
    """online training (fresh samples every step, as the cache is trained during rendering)"""
    c = NeuralRadianceCache(ctx)  # full size: 16 levels x 2^19 entries
    test = random_features(8192, 999)
    tt = _field(test)
    before = ((c.infer(test) - tt).abs().mean() / tt.abs().mean()).item()
    losses = []
    for step in range(400):
        feats = random_features(65536, 1000 + step)
        losses.append(c.train_step(feats, _field(feats)))
    after = ((c.infer(test) - tt).abs().mean() / tt.abs().mean()).item()
    print("loss", losses[0], "->", losses[-1], "held-out relative error", before, "->", after)
    assert losses[-1] < 0.05 * losses[0]
    # online Adam at lr 1e-2 is noisy: 400 steps land between 0.035 and 0.09 across runs
    assert after < 0.15 and after < 0.2 * before
    c.close()
