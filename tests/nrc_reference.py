"""PyTorch reference of the neural radiance cache (test helper, not product code): the same hash-grid
+ spherical-harmonics encoding and the same bias-free 80-64x5-3 ReLU MLP, evaluated from the
library's FP32 master parameters, for checking the CUDA kernels' predictions and gradients."""
from __future__ import annotations

import math

import numpy as np
import torch

IN, HID, OUTP = 80, 64, 16
LAYERS = [(IN, HID)] + [(HID, HID)] * 4 + [(HID, OUTP)]


def split_weights(flat: torch.Tensor):
    out, off = [], 0
    for k, n in LAYERS:
        out.append(flat[off: off + k * n].view(k, n))
        off += k * n
    return out


def bf16(x: torch.Tensor) -> torch.Tensor:
    return x.to(torch.bfloat16).to(x.dtype)


def sh4(d: torch.Tensor) -> torch.Tensor:
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    xx, yy, zz = x * x, y * y, z * z
    return torch.stack([
        torch.full_like(x, 0.28209479177387814), -0.48860251190291987 * y, 0.48860251190291987 * z,
        -0.48860251190291987 * x, 1.0925484305920792 * x * y, -1.0925484305920792 * y * z,
        0.31539156525252005 * (3 * zz - 1), -1.0925484305920792 * x * z, 0.5462742152960396 * (xx - yy),
        -0.5900435899266435 * y * (3 * xx - yy), 2.890611442640554 * x * y * z,
        -0.4570457994644658 * y * (5 * zz - 1), 0.3731763325901154 * z * (5 * zz - 3),
        -0.4570457994644658 * x * (5 * zz - 1), 1.445305721320277 * z * (xx - yy),
        -0.5900435899266435 * x * (xx - 3 * yy)], dim=1)


def encode(feats: torch.Tensor, grid: torch.Tensor, res: list[int], table: int, smin, smax,
           half_grid: bool = True) -> torch.Tensor:
    """feats [N,13] fp32; grid [levels*table*2] (fp32 master; rounded to fp16 like the GPU copy)."""
    dev = feats.device
    smin_t = torch.tensor(smin, dtype=torch.float32, device=dev)
    sinv = 1.0 / (torch.tensor(smax, dtype=torch.float32, device=dev) - smin_t)
    p = ((feats[:, 0:3].float() - smin_t) * sinv).clamp(0, 1)
    g = grid.view(len(res), table, 2)
    if half_grid:
        g = g.to(torch.float16).to(grid.dtype)
    cols = []
    for l, r in enumerate(res):
        x = p * float(r)
        fl = torch.floor(x).clamp(max=float(r - 1))
        c = fl.to(torch.int64)
        f = (x - fl).to(grid.dtype)
        dense = (r + 1) ** 3 <= table
        acc = torch.zeros((feats.shape[0], 2), dtype=grid.dtype, device=dev)
        for k in range(8):
            o = torch.tensor([k & 1, (k >> 1) & 1, (k >> 2) & 1], device=dev)
            cc = c + o
            w = torch.where(o.bool(), f, 1 - f).prod(dim=1)
            if dense:
                idx = cc[:, 0] + cc[:, 1] * (r + 1) + cc[:, 2] * (r + 1) ** 2
            else:
                u = cc.to(torch.int64) & 0xFFFFFFFF
                idx = (u[:, 0] ^ ((u[:, 1] * 2654435761) & 0xFFFFFFFF) ^ ((u[:, 2] * 805459861) & 0xFFFFFFFF)) & (table - 1)
            acc = acc + w[:, None] * g[l].index_select(0, idx)
        cols.append(acc)
    grid_feats = torch.cat(cols, dim=1)
    rest = torch.cat([sh4(feats[:, 3:6].float()), sh4(feats[:, 6:9].float()), feats[:, 9:13].float()], dim=1)
    pad = torch.zeros((feats.shape[0], IN - 32 - rest.shape[1]), device=dev)
    return torch.cat([grid_feats, rest.to(grid.dtype), pad.to(grid.dtype)], dim=1)


def forward(X: torch.Tensor, weights: list[torch.Tensor], emulate_bf16: bool = True) -> torch.Tensor:
    h = bf16(X) if emulate_bf16 else X
    for l, w in enumerate(weights):
        wq = bf16(w) if emulate_bf16 else w
        z = h @ wq
        if l < len(weights) - 1:
            h = torch.relu(z)
            if emulate_bf16:
                h = bf16(h)
        else:
            h = z
    return h[:, :3]


def relative_l2(y: torch.Tensor, t: torch.Tensor) -> torch.Tensor:
    return ((y - t) ** 2 / (y.detach() ** 2 + 0.01)).mean()


def random_features(n: int, seed: int, device="cuda") -> torch.Tensor:
    g = torch.Generator().manual_seed(seed)
    pos = torch.rand((n, 3), generator=g) * 2 - 1
    d = torch.randn((n, 3), generator=g)
    d = d / d.norm(dim=1, keepdim=True)
    nn = torch.randn((n, 3), generator=g)
    nn = nn / nn.norm(dim=1, keepdim=True)
    rough = torch.rand((n, 1), generator=g)
    alb = torch.rand((n, 3), generator=g)
    return torch.cat([pos, d, nn, rough, alb], dim=1).float().to(device)


def level_resolutions(levels=16, base=16, maxres=2048) -> list[int]:
    growth = np.float32(math.exp((math.log(np.float32(maxres)) - math.log(np.float32(base))) / (levels - 1)))
    out = []
    for l in range(levels):
        r = np.float32(base)
        for _ in range(l):
            r = np.float32(r * growth)
        out.append(int(r))
    return out
