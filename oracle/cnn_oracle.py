"""CPU (numpy FP64) restatement of the learned warm start's network, used as
the checker of the GPU forward/backward kernels.  TEST INFRASTRUCTURE ONLY.

Network: 6 conv3x3 layers ('same' zero padding, dilations 1, 2, 4, 8, 2, 1),
channels 3 -> 32 -> 32 -> 32 -> 32 -> 32 -> 4, ReLU after layers 1-5; loss = mean over (batch, 4 outputs,
31 x 31 interior nodes) of (prediction - target)^2.  Parameters are one flat
vector: per layer W [Cout][Cin][3][3] then b [Cout].

With bf16=True the oracle rounds exactly where the GPU stores BF16 (inputs,
weights, hidden activations, layer gradients) and computes in FP64
otherwise, so GPU results agree up to FP32 accumulation order.
"""
import numpy as np

CH = [3, 32, 32, 32, 32, 32, 4]
DIL = [1, 2, 4, 8, 2, 1]
H = W = 33


def param_shapes():
    out = []
    for l in range(6):
        out.append(((CH[l + 1], CH[l], 3, 3), (CH[l + 1],)))
    return out


def param_count():
    return sum(int(np.prod(w)) + int(np.prod(b)) for w, b in param_shapes())


def unpack(params):
    layers, off = [], 0
    for ws, bs in param_shapes():
        nw, nb = int(np.prod(ws)), int(np.prod(bs))
        layers.append((params[off:off + nw].reshape(ws), params[off + nw:off + nw + nb]))
        off += nw + nb
    return layers


def pack(grads):
    return np.concatenate([np.concatenate([gw.ravel(), gb.ravel()]) for gw, gb in grads])


def bf16(x):
    """Round to bfloat16 (nearest even), returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def conv(x, w, b=None, d=1):
    """x [B][Cin][H][W], w [Cout][Cin][3][3] -> [B][Cout][H][W] ('same', dilation d)."""
    xp = np.pad(x, ((0, 0), (0, 0), (d, d), (d, d)))
    out = np.zeros((x.shape[0], w.shape[0], x.shape[2], x.shape[3]))
    for ty in range(3):
        for tx in range(3):
            sl = xp[:, :, ty * d:ty * d + x.shape[2], tx * d:tx * d + x.shape[3]]
            out += np.einsum("bchw,oc->bohw", sl, w[:, :, ty, tx])
    if b is not None:
        out += b[None, :, None, None]
    return out


def conv_grads(x, w, g, d=1):
    """Gradients of conv(x, w, d) wrt w, b and x given the output gradient g."""
    xp = np.pad(x, ((0, 0), (0, 0), (d, d), (d, d)))
    gw = np.zeros_like(w)
    for ty in range(3):
        for tx in range(3):
            sl = xp[:, :, ty * d:ty * d + x.shape[2], tx * d:tx * d + x.shape[3]]
            gw[:, :, ty, tx] = np.einsum("bohw,bchw->oc", g, sl)
    gb = g.sum(axis=(0, 2, 3))
    # dx = conv(g, flipped/transposed w) at the same dilation
    wt = np.transpose(w[:, :, ::-1, ::-1], (1, 0, 2, 3))
    gx = conv(g, wt, None, d)
    return gw, gb, gx


def forward(params, feats, bf16_mode=True, keep=False):
    r = bf16 if bf16_mode else (lambda a: np.asarray(a, dtype=np.float64))
    layers = unpack(np.asarray(params, dtype=np.float64))
    h = r(feats)
    acts = [h]
    for l, (w, b) in enumerate(layers):
        z = conv(h, r(w), np.asarray(b, dtype=np.float64), DIL[l])
        if l < 5:
            h = r(np.maximum(z, 0.0))
        else:
            h = z
        acts.append(h)
    return (h, acts) if keep else h


def loss_and_grads(params, feats, targets, bf16_mode=True):
    r = bf16 if bf16_mode else (lambda a: np.asarray(a, dtype=np.float64))
    layers = unpack(np.asarray(params, dtype=np.float64))
    pred, acts = forward(params, feats, bf16_mode, keep=True)
    B = feats.shape[0]
    scale = 1.0 / (B * 4 * (H - 2) * (W - 2))
    mask = np.zeros((H, W))
    mask[1:-1, 1:-1] = 1.0
    d = (pred - targets) * mask
    loss = float((d * d).sum() * scale)
    g = r(2.0 * scale * d)
    grads = [None] * 6
    for l in range(5, -1, -1):
        w, _ = layers[l]
        gw, gb, gx = conv_grads(acts[l], r(w), g, DIL[l])
        grads[l] = (gw, gb)
        if l > 0:
            g = r(gx * (acts[l] > 0))
    return loss, pack(grads)
