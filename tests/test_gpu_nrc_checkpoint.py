"""Radiance-cache checkpoints (vkg_nrc_save / vkg_nrc_load): a trained cache saved and loaded into a
fresh cache gives the same parameters, Adam moments, step count and predictions bit for bit (saving
the loaded cache writes the same bytes), and training continues from the loaded state as from the
original (the hash-grid gradients are summed with atomics, so two training runs agree to rounding,
not bit for bit); a corrupted payload, a truncated file and a cache with another grid layout are
refused."""
import ctypes as C

import numpy as np
import pytest
import torch

from nrc_reference import random_features
from vierkant_gb300 import _lib
from vierkant_gb300.nrc import NeuralRadianceCache

pytestmark = pytest.mark.gpu


def _small_config():
    cfg = NeuralRadianceCache.default_config()
    cfg.log2_table_size = 14
    return cfg


def _params(cache):
    i = cache.info()
    mlp = torch.empty(i.num_mlp_params, dtype=torch.float32, device="cuda")
    grid = torch.empty(i.num_grid_params, dtype=torch.float32, device="cuda")
    rt = _lib_cudart()
    rt.cudaMemcpy(C.c_void_p(mlp.data_ptr()), C.c_void_p(i.d_mlp_params), C.c_size_t(4 * i.num_mlp_params), 3)
    rt.cudaMemcpy(C.c_void_p(grid.data_ptr()), C.c_void_p(i.d_grid_params), C.c_size_t(4 * i.num_grid_params), 3)
    return mlp.cpu().numpy(), grid.cpu().numpy(), i.step


def _lib_cudart():
    from vierkant_gb300.raytracing import _cudart
    return _cudart()


def _train(cache, steps, seed):
    for k in range(steps):
        x = random_features(8192, seed=seed + k)
        g = torch.Generator(device="cuda").manual_seed(seed + k)
        t = torch.rand((8192, 3), device="cuda", generator=g)
        cache.train_step(x, t)
    torch.cuda.synchronize()


def test_checkpoint_round_trip_and_resume(ctx, tmp_path):
    a = NeuralRadianceCache(ctx, _small_config())
    _train(a, 5, 10)
    path = tmp_path / "cache.vkgnrc"
    a.save(path)
    b = NeuralRadianceCache(ctx, _small_config())
    b.load(path)
    ma, ga, sa = _params(a)
    mb, gb, sb = _params(b)
    assert sa == sb == 5
    assert ma.tobytes() == mb.tobytes() and ga.tobytes() == gb.tobytes()
    q = random_features(4096, seed=99)
    assert torch.equal(a.infer(q), b.infer(q))
    # the whole training state came along, Adam moments included: saving it again gives the same file
    path2 = tmp_path / "again.vkgnrc"
    b.save(path2)
    assert path.read_bytes() == path2.read_bytes()
    # and training continues from it as from the original
    _train(a, 3, 50)
    _train(b, 3, 50)
    ma, ga, sa = _params(a)
    mb, gb, sb = _params(b)
    assert sa == sb == 8
    assert np.allclose(ma, mb, rtol=0, atol=2e-3) and np.allclose(ga, gb, rtol=0, atol=2e-3)
    pa, pb = a.infer(q), b.infer(q)
    assert (pa - pb).abs().max().item() <= 1e-2 * max(1.0, pa.abs().max().item())
    assert a.info().kernel_error == 0 and b.info().kernel_error == 0
    a.close()
    b.close()


def test_checkpoint_rejects_bad_files(ctx, tmp_path):
    a = NeuralRadianceCache(ctx, _small_config())
    _train(a, 2, 3)
    path = tmp_path / "cache.vkgnrc"
    a.save(path)
    raw = bytearray(path.read_bytes())
    hdr = np.frombuffer(bytes(raw[:128]), np.uint8)
    assert bytes(hdr[:8]) == b"VKGNRC01"
    bad = tmp_path / "flipped.vkgnrc"
    raw2 = bytearray(raw)
    raw2[128 + 1000] ^= 0x40
    bad.write_bytes(bytes(raw2))
    with pytest.raises(_lib.VkgError, match="checksum"):
        a.load(bad)
    short = tmp_path / "short.vkgnrc"
    short.write_bytes(bytes(raw[:-4]))
    with pytest.raises(_lib.VkgError):
        a.load(short)
    other = NeuralRadianceCache(ctx, NeuralRadianceCache.default_config())  # 2^19 entries per level
    with pytest.raises(_lib.VkgError, match="layout"):
        other.load(path)
    with pytest.raises(_lib.VkgError):
        a.load(tmp_path / "missing.vkgnrc")
    other.close()
    a.close()
