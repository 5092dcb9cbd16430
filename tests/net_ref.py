"""PyTorch CPU (FP32) restatement of the warm-start network, for checks only.

Layer table, parameter layout and tensor orders follow include/fsim.h
(fsim_net_*): flat FP32 parameters, per layer weights [tap][cout][cin] (tap =
(kd*3 + kh)*3 + kw) then bias [cout]; the 2x2x2 stride-2 down-convolutions are
pointwise layers over space-to-depth channels (sub*C + c, sub = sd*4 + sh*2 +
sw); head weight [16], bias [1].  Inputs [n, d, h, w, 4].
"""
from __future__ import annotations

import torch
import torch.nn.functional as F

SPEC = [(27, 16, 16), (27, 16, 16), (1, 128, 32), (27, 32, 32), (27, 32, 32), (1, 256, 64),
        (27, 64, 64), (27, 64, 64), (1, 512, 64), (27, 64, 64), (27, 64, 64), (27, 128, 64),
        (27, 64, 64), (27, 96, 32), (27, 32, 32), (27, 48, 16), (27, 16, 16)]


def layout():
    off = 0
    out = []
    for taps, cin, cout in SPEC:
        w = off
        off += taps * cin * cout
        b = off
        off += cout
        out.append((w, b))
    head_w = off
    head_b = off + 16
    return out, head_w, head_b, off + 17


def num_params() -> int:
    return layout()[3]


class _RoundBF16(torch.autograd.Function):
    """Round to BF16 where the kernels store a BF16 tensor: the value going
    forward and the gradient coming back."""

    @staticmethod
    def forward(ctx, x):
        return x.bfloat16().float()

    @staticmethod
    def backward(ctx, g):
        return g.bfloat16().float()


def forward(theta: torch.Tensor, x: torch.Tensor, out_scale: float = 1.0, bf16: bool = False) -> torch.Tensor:
    offs, hw, hb, total = layout()
    assert theta.numel() == total

    def wb(l):
        taps, cin, cout = SPEC[l]
        w0, b0 = offs[l]
        w = theta[w0:w0 + taps * cin * cout].view(taps, cout, cin)
        return w, theta[b0:b0 + cout]

    rnd = _RoundBF16.apply if bf16 else (lambda t: t)

    def conv(l, inp):
        w, b = wb(l)
        wt = w.permute(1, 2, 0).reshape(w.shape[1], w.shape[2], 3, 3, 3)
        return rnd(F.relu(F.conv3d(inp, wt, b, padding=1)))

    def down(l, inp):
        w, b = wb(l)
        C = inp.shape[1]
        wt = w[0].view(w.shape[1], 8, C).permute(0, 2, 1).reshape(w.shape[1], C, 2, 2, 2)
        return rnd(F.relu(F.conv3d(rnd(inp), wt, b, stride=2)))

    def up(t):
        return rnd(F.interpolate(t, scale_factor=2, mode="trilinear", align_corners=False))

    def cat(a, b):
        return rnd(torch.cat([a, b], 1))

    x0 = x.permute(0, 4, 1, 2, 3)
    x0 = rnd(torch.cat([x0, torch.zeros(x0.shape[0], 12, *x0.shape[2:], dtype=x0.dtype)], 1))
    a0 = conv(0, x0)
    e0 = conv(1, a0)
    x1 = down(2, e0)
    a1 = conv(3, x1)
    e1 = conv(4, a1)
    x2 = down(5, e1)
    a2 = conv(6, x2)
    e2 = conv(7, a2)
    x3 = down(8, e2)
    a3 = conv(9, x3)
    b3 = conv(10, a3)
    c2 = conv(11, cat(up(b3), e2))
    d2 = conv(12, c2)
    c1 = conv(13, cat(up(d2), e1))
    d1 = conv(14, c1)
    c0 = conv(15, cat(up(d1), e0))
    d0 = conv(16, c0)
    out = torch.einsum("ncdhw,c->ndhw", d0, theta[hw:hw + 16]) + theta[hb]
    return out_scale * out


def operator(e: torch.Tensor, m: torch.Tensor, solid: torch.Tensor) -> torch.Tensor:
    """The solver's 7-point operator on fluid voxels (out-of-volume neighbours solid)."""
    e = e * m
    pe = F.pad(e, (1, 1, 1, 1, 1, 1))
    ps = F.pad(solid, (1, 1, 1, 1, 1, 1), value=1.0)
    D, H, W = e.shape[1:]
    nb = torch.zeros_like(e)
    ns = torch.zeros_like(e)
    for dd, dh, dw in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
        sl = (slice(None), slice(1 + dd, 1 + dd + D), slice(1 + dh, 1 + dh + H), slice(1 + dw, 1 + dw + W))
        nb = nb + pe[sl]
        ns = ns + (1.0 - ps[sl])
    return m * (ns * e - nb)


def loss_and_grad(theta_np, x_np, t_np, m_np, out_scale: float = 1.0, l2_weight: float = 0.1, bf16: bool = True):
    """Loss of fsim_net_backward: mean over samples of ||A e|| / ||b|| +
    l2_weight ||e|| / ||target|| (b = input channel 0 as the kernels store it,
    in BF16)."""
    theta = torch.tensor(theta_np, dtype=torch.float32, requires_grad=True)
    x = torch.tensor(x_np, dtype=torch.float32)
    t = torch.tensor(t_np, dtype=torch.float32)
    m = torch.tensor(m_np.astype("float32"))
    out = forward(theta, x, out_scale, bf16=bf16)
    e = (out - t) * m
    r = operator(e, m, x[..., 2])
    b = x[..., 0].bfloat16().float() * m
    tm = t * m
    dims = (1, 2, 3)
    loss = (r.pow(2).sum(dims).sqrt() / b.pow(2).sum(dims).sqrt()
            + l2_weight * e.pow(2).sum(dims).sqrt() / tm.pow(2).sum(dims).sqrt()).mean()
    loss.backward()
    return float(loss.detach()), out.detach().numpy(), theta.grad.numpy()
