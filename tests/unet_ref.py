"""numpy restatement of the U-Net of vulkanfem_gb300/csrc/unet.cu (the oracle
for its forward and backward kernels).

BF16 rounding is applied where the CUDA kernels store BF16 (inputs, weights,
conv outputs, pooled and concatenated activations, the relu-masked output
gradient); every sum is carried in float64, so the comparison isolates the
kernels' FP32-accumulation rounding.  Layout: channels-last [z, y, x, c].
"""
import numpy as np

CIN = (16, 16, 32, 64, 192, 96, 48, 16)
COUT = (16, 32, 64, 128, 64, 32, 16, 16)
RELU = (1, 1, 1, 1, 1, 1, 1, 0)


ROUND = True  # False: plain float64 everywhere (finite-difference checks of the restatement itself)


def bf(x):
    """Round float64/float32 to bfloat16 (round to nearest even), returned as float64."""
    if not ROUND:
        return np.asarray(x, dtype=np.float64).copy()
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32).astype(np.float64)


def param_layout():
    off, out = 0, []
    for ci, co in zip(CIN, COUT):
        w = (off, off + 27 * ci * co)
        off = w[1]
        b = (off, off + co)
        off = b[1]
        out.append((w, b))
    return out, off


def init_params(seed=0):
    lay, n = param_layout()
    rng = np.random.default_rng(seed)
    p = np.zeros(n, np.float32)
    for (w0, w1), (b0, b1) in lay:
        l = lay.index(((w0, w1), (b0, b1)))
        fan_in = 27 * CIN[l]
        p[w0:w1] = rng.standard_normal(w1 - w0) * np.sqrt(2.0 / fan_in)
        p[b0:b1] = 0.0
    return p


def unpack(p):
    lay, _ = param_layout()
    W, B = [], []
    for l, ((w0, w1), (b0, b1)) in enumerate(lay):
        W.append(np.asarray(p[w0:w1], np.float64).reshape(27, CIN[l], COUT[l]))
        B.append(np.asarray(p[b0:b1], np.float64))
    return W, B


def _taps():
    return [(t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1) for t in range(27)]


def conv(x, W, b=None):
    """x [n,n,n,Cin], W [27,Cin,Cout] -> [n,n,n,Cout] (zero padding)."""
    n = x.shape[0]
    xp = np.zeros((n + 2, n + 2, n + 2, x.shape[3]))
    xp[1:-1, 1:-1, 1:-1] = x
    out = np.zeros((n, n, n, W.shape[2]))
    for t, (dx, dy, dz) in enumerate(_taps()):
        sl = xp[1 + dz:1 + dz + n, 1 + dy:1 + dy + n, 1 + dx:1 + dx + n]
        out += sl @ W[t]
    if b is not None:
        out += b
    return out


def conv_wgrad(x, g):
    """dW[t] = sum_v x[v + off(t)] g[v]^T."""
    n = x.shape[0]
    xp = np.zeros((n + 2, n + 2, n + 2, x.shape[3]))
    xp[1:-1, 1:-1, 1:-1] = x
    dW = np.zeros((27, x.shape[3], g.shape[3]))
    for t, (dx, dy, dz) in enumerate(_taps()):
        sl = xp[1 + dz:1 + dz + n, 1 + dy:1 + dy + n, 1 + dx:1 + dx + n]
        dW[t] = sl.reshape(-1, x.shape[3]).T @ g.reshape(-1, g.shape[3])
    return dW


def conv_dgrad(g, W):
    """dX[v] = sum_t W[t] g[v - off(t)]  (flipped, transposed weights)."""
    Wt = W[::-1].transpose(0, 2, 1)
    return conv(g, Wt)


def pool(x):
    n = x.shape[0] // 2
    return x.reshape(n, 2, n, 2, n, 2, -1).mean(axis=(1, 3, 5))


def pool_bwd(g):
    return np.repeat(np.repeat(np.repeat(g, 2, 0), 2, 1), 2, 2) / 8.0


def up(x):
    return np.repeat(np.repeat(np.repeat(x, 2, 0), 2, 1), 2, 2)


def up_bwd(g):
    n = g.shape[0] // 2
    return g.reshape(n, 2, n, 2, n, 2, -1).sum(axis=(1, 3, 5))


def forward(p, x_in):
    """Returns (y, cache). x_in [n,n,n,16]."""
    W, B = unpack(p)
    Wb = [bf(w) for w in W]
    c = {}
    c["x"] = x = bf(x_in)
    relu = lambda a: np.maximum(a, 0.0)
    c["e0"] = e0 = bf(relu(conv(x, Wb[0], B[0])))
    c["p1"] = p1 = bf(pool(e0))
    c["e1"] = e1 = bf(relu(conv(p1, Wb[1], B[1])))
    c["p2"] = p2 = bf(pool(e1))
    c["e2"] = e2 = bf(relu(conv(p2, Wb[2], B[2])))
    c["p3"] = p3 = bf(pool(e2))
    c["e3"] = e3 = bf(relu(conv(p3, Wb[3], B[3])))
    c["c2"] = c2 = np.concatenate([up(e3), e2], axis=3)
    c["d2"] = d2 = bf(relu(conv(c2, Wb[4], B[4])))
    c["c1"] = c1 = np.concatenate([up(d2), e1], axis=3)
    c["d1"] = d1 = bf(relu(conv(c1, Wb[5], B[5])))
    c["c0"] = c0 = np.concatenate([up(d1), e0], axis=3)
    c["d0"] = d0 = bf(relu(conv(c0, Wb[6], B[6])))
    c["y"] = y = conv(d0, Wb[7], B[7])
    c["Wb"] = Wb
    return y, c


def loss_and_grads(p, x_in, target, mask):
    """Masked MSE over channels 0..2 and the parameter gradient (packed)."""
    y, c = forward(p, x_in)
    Wb = c["Wb"]
    cnt = 3.0 * mask.sum()
    d = (y[..., :3] - target) * mask[..., None]
    loss = float((d * (y[..., :3] - target)).sum() / cnt)
    gy = np.zeros_like(y)
    gy[..., :3] = 2.0 * d / cnt
    lay, n = param_layout()
    grads = np.zeros(n)

    def layer_bwd(l, inp, out, g):
        gm = bf(g * (out > 0) if RELU[l] else g)
        (w0, w1), (b0, b1) = lay[l]
        grads[b0:b1] += gm.reshape(-1, gm.shape[3]).sum(axis=0)
        grads[w0:w1] += conv_wgrad(inp, gm).reshape(-1)
        return conv_dgrad(gm, Wb[l])

    gd0 = layer_bwd(7, c["d0"], None, gy)
    gc0 = layer_bwd(6, c["c0"], c["d0"], gd0)
    gd1 = up_bwd(gc0[..., :32])
    ge0 = gc0[..., 32:].copy()
    gc1 = layer_bwd(5, c["c1"], c["d1"], gd1)
    gd2 = up_bwd(gc1[..., :64])
    ge1 = gc1[..., 64:].copy()
    gc2 = layer_bwd(4, c["c2"], c["d2"], gd2)
    ge3 = up_bwd(gc2[..., :128])
    ge2 = gc2[..., 128:].copy()
    gp3 = layer_bwd(3, c["p3"], c["e3"], ge3)
    ge2 += pool_bwd(gp3)
    gp2 = layer_bwd(2, c["p2"], c["e2"], ge2)
    ge1 += pool_bwd(gp2)
    gp1 = layer_bwd(1, c["p1"], c["e1"], ge1)
    ge0 += pool_bwd(gp1)
    layer_bwd(0, c["x"], c["e0"], ge0)
    return loss, grads, y
