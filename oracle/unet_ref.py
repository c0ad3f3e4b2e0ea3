"""CPU oracle of the learned preconditioner -- TEST INFRASTRUCTURE ONLY.

An FP64 restatement, in torch on the CPU, of the network the GPU applies
(plask_gb300/csrc/unet.cu, unet_ops.cu): the same layers, the same input
features, 2x2x2 average pooling with ceil extents (missing children count as
zero), upsampling by copy, the output head, the correction direction
v = D^-1/2 u with its A-norm optimal weight, and the loss
1 - (v, r)^2 / ((v, A v)(e, A e)).  Tensors the GPU stores in BF16 are rounded to
BF16 at the same points (straight through in the backward pass), so autograd
gives the gradient of the same computation the GPU's hand-written backward
kernels differentiate.  The system matrix A is the oracle's own assembled,
Dirichlet-eliminated matrix (oracle/fem3d.py).
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn.functional as Fn

LAYERS = [("lift", 16, 16, 1), ("enc1", 16, 32, 27), ("enc2", 32, 48, 27), ("enc3", 48, 64, 27),
          ("bott", 64, 64, 27), ("proj2", 64, 48, 1), ("dec2", 48, 48, 27), ("proj1", 48, 32, 1),
          ("dec1", 32, 32, 27), ("proj0", 32, 16, 1)]
HEAD = 16


def split_weights(flat):
    """Flat FP32 weights -> list of torch conv weights [cout, cin, kz, ky, kx] and the head."""
    out, o = [], 0
    for _, cin, cout, taps in LAYERS:
        n = taps * cout * cin
        w = np.asarray(flat[o:o + n], np.float64).reshape(taps, cout, cin)
        o += n
        if taps == 27:
            w = w.reshape(3, 3, 3, cout, cin).transpose(3, 4, 0, 1, 2)  # tap = dx + 3 dy + 9 dz
        else:
            w = w.reshape(cout, cin, 1, 1, 1)
        out.append(w)
    head = np.asarray(flat[o:o + HEAD], np.float64)
    return out, head


def bf16_np(a):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return (r.astype(np.uint32) << 16).astype(np.uint32).view(np.float32).astype(np.float64)


def _bf16(t):
    return t + (t.to(torch.bfloat16).to(t.dtype) - t).detach()


def _pool(x):
    _, _, d, h, w = x.shape
    x = Fn.pad(x, (0, w % 2, 0, h % 2, 0, d % 2))
    return Fn.avg_pool3d(x, 2, 2)


def _up(x, shape):
    y = x.repeat_interleave(2, 2).repeat_interleave(2, 3).repeat_interleave(2, 4)
    return y[:, :, : shape[0], : shape[1], : shape[2]]


def _conv(x, w):
    k = w.shape[-1]
    return Fn.conv3d(x, w, padding=k // 2)


def features(axes, kxy, kz, minv):
    """Input channels 1..4 per node (k_unet_features): FP32 conductance sums of the node's elements.

    kxy, kz: FP32 per element, canonical (ne2, ne1, ne0); minv: FP32 per node (n2, n1, n0)."""
    x0, x1, x2 = (np.asarray(a, np.float64) for a in axes)
    h = [np.diff(a).astype(np.float32) for a in (x0, x1, x2)]
    r = [(1.0 / np.diff(a)).astype(np.float32) for a in (x0, x1, x2)]
    n2, n1, n0 = minv.shape
    sx = np.zeros((n2, n1, n0), np.float32)
    sy = np.zeros_like(sx)
    sz = np.zeros_like(sx)
    dz = h[2][:, None, None]
    dy = h[1][None, :, None]
    dx = h[0][None, None, :]
    X = ((kxy * dy) * dz) * r[0][None, None, :]
    Y = ((kxy * dx) * dz) * r[1][None, :, None]
    Z = ((kz * dx) * dy) * r[2][:, None, None]
    for c in range(8):
        ci, cj, ck = c & 1, (c >> 1) & 1, c >> 2
        sl = (slice(ck, ck + n2 - 1), slice(cj, cj + n1 - 1), slice(ci, ci + n0 - 1))
        sx[sl] += X.astype(np.float32)
        sy[sl] += Y.astype(np.float32)
        sz[sl] += Z.astype(np.float32)
    tiny = np.float32(1e-30)
    f = np.zeros((16,) + minv.shape)
    f[1] = np.clip(np.float32(0.25) * np.log((sx + tiny) / (sz + tiny)), -4, 4)
    f[2] = np.clip(np.float32(0.25) * np.log((sy + tiny) / (sz + tiny)), -4, 4)
    f[3] = (minv == 0).astype(np.float32)
    f[4] = np.clip(np.float32(0.1) * np.log10(sx + sy + sz + tiny), -4, 4)
    return bf16_np(f.astype(np.float32))


def forward(weights, head, feat, r, minv):
    """Network direction v = D^-1/2 u for residual r (n2, n1, n0); returns torch tensors (v, u, W, H)."""
    N = r.size
    sig2 = float(np.sum(r.astype(np.float64) * minv.astype(np.float64) * r.astype(np.float64))) / N
    sigma = np.sqrt(sig2)
    f0 = bf16_np((np.sqrt(minv) * r * np.float32(1.0 / sigma)).astype(np.float32))
    x = torch.tensor(np.concatenate([f0[None], feat[1:]], 0)[None])
    W = [torch.tensor(w, requires_grad=True) for w in weights]
    H = torch.tensor(head, requires_grad=True)
    s0 = x.shape[2:]
    x0 = _bf16(torch.relu(_conv(x, W[0])))
    pool0 = _bf16(_pool(x0))
    x1 = _bf16(torch.relu(_conv(pool0, W[1])))
    s1 = x1.shape[2:]
    pool1 = _bf16(_pool(x1))
    x2 = _bf16(torch.relu(_conv(pool1, W[2])))
    s2 = x2.shape[2:]
    pool2 = _bf16(_pool(x2))
    x3 = _bf16(torch.relu(_conv(pool2, W[3])))
    x3b = _bf16(torch.relu(_conv(x3, W[4])))
    p2 = _bf16(_conv(x3b, W[5]))
    y2 = _bf16(torch.relu(_conv(_bf16(x2 + _up(p2, s2)), W[6])))
    p1 = _bf16(_conv(y2, W[7]))
    y1 = _bf16(torch.relu(_conv(_bf16(x1 + _up(p1, s1)), W[8])))
    p0 = _bf16(_conv(y1, W[9]))
    q = x0 + _up(p0, s0)
    u = torch.einsum("c,bcdhw->bdhw", H, q)[0]
    m = torch.tensor(minv.astype(np.float64))
    v = torch.where(m > 0, torch.sqrt(m) * u, torch.zeros_like(u))
    return v, u, W, H


def loss_and_grad(flat, feat, r, minv, e, A_canonical):
    """Loss 1 - (v, r)^2 / ((v, A v)(e, r)) and its gradient w.r.t. the flat weights;
    also the preconditioned residual z = M^-1 r + ((v, r) / (v, A v)) v.

    r = A e as the GPU computed it; A_canonical: scipy sparse matrix in canonical node order."""
    weights, head = split_weights(flat)
    v, u, W, H = forward(weights, head, feat, r, minv)
    vv = v.reshape(-1)
    rt = torch.tensor(r.ravel().astype(np.float64))
    ev = torch.tensor(e.ravel().astype(np.float64))
    Acoo = A_canonical.tocoo()
    A = torch.sparse_coo_tensor(np.vstack([Acoo.row, Acoo.col]), Acoo.data, A_canonical.shape)
    a = vv @ rt
    b = vv @ torch.sparse.mm(A, vv[:, None])[:, 0]
    E = float(ev @ rt)
    loss = 1.0 - a * a / (b * E)
    z = torch.tensor(minv.ravel().astype(np.float64)) * rt + (a / b) * vv
    loss.backward()
    g = []
    for (_, cin, cout, taps), w in zip(LAYERS, W):
        gw = w.grad.numpy()
        if taps == 27:
            gw = gw.transpose(2, 3, 4, 0, 1).reshape(27, cout, cin)
        else:
            gw = gw.reshape(1, cout, cin)
        g.append(gw.ravel())
    g.append(H.grad.numpy())
    return float(loss.detach()), np.concatenate(g), z.detach().numpy()
