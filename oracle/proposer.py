"""CPU oracle of the learned pose proposer (merge_fusion_gb300/csrc/
kifi_proposer.cu) -- test infrastructure only.

The same network, parameter layout and loss in float64 numpy.  With
``quantize=True`` values are rounded to BF16 at exactly the points where the
GPU stores BF16 (im2col columns, weights, activations, the pooled features,
the BF16 copies of the gradients the backward GEMMs read), so the GPU's
results differ from it only by FP32 accumulation order.  With
``quantize=False`` it is the exact float64 network, whose backward pass is
checked against finite differences.  The proposer has no counterpart in the
reference; this oracle is its own CPU forward/backward."""
import numpy as np

CONVS = [  # (C_in, C_out, H_in, W_in, H_out, W_out, K padded)
    (2, 32, 60, 80, 30, 40, 32),
    (32, 64, 30, 40, 15, 20, 288),
    (64, 64, 15, 20, 8, 10, 576),
    (64, 128, 8, 10, 4, 5, 576),
]
FC1, OUT, OUT_PAD = 64, 6, 16
SHAPES = [(32, 32), (32,), (64, 288), (64,), (64, 576), (64,), (128, 576), (128,), (64, 128), (64,),
          (16, 64), (16,)]


def layout():
    """(offset, shape) per parameter tensor and the total length."""
    out, total = [], 0
    for shp in SHAPES:
        n = int(np.prod(shp))
        out.append((total, shp))
        total += (n + 7) // 8 * 8
    return out, total


def trainable_mask():
    lay, total = layout()
    m = np.zeros(total, bool)
    for t, (off, shp) in enumerate(lay):
        n = int(np.prod(shp))
        idx = np.arange(n)
        on = np.ones(n, bool)
        if t == 0:
            on = (idx % 32) < 18
        if t == 10:
            on = (idx // FC1) < OUT
        if t == 11:
            on = idx < OUT
        m[off:off + n] = on
    return m


def unpack(vec):
    lay, _ = layout()
    return [np.asarray(vec[o:o + int(np.prod(s))], np.float64).reshape(s) for o, s in lay]


def pack(tensors):
    lay, total = layout()
    v = np.zeros(total, np.float64)
    for (o, s), t in zip(lay, tensors):
        v[o:o + int(np.prod(s))] = np.asarray(t, np.float64).reshape(-1)
    return v


def bf16(x):
    """Round to the nearest BF16 (ties to even), as float64."""
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def im2col(x, cfg):
    cin, _, h, w, ho, wo, kp = cfg
    b = x.shape[0]
    xp = np.zeros((b, h + 2, w + 2, cin))
    xp[:, 1:h + 1, 1:w + 1, :] = x
    col = np.zeros((b, ho, wo, kp))
    for ky in range(3):
        for kx in range(3):
            tap = ky * 3 + kx
            col[..., tap * cin:(tap + 1) * cin] = xp[:, ky:ky + 2 * ho:2, kx:kx + 2 * wo:2, :]
    return col.reshape(b * ho * wo, kp)


def col2im(dcol, cfg, b):
    cin, _, h, w, ho, wo, kp = cfg
    dxp = np.zeros((b, h + 2, w + 2, cin))
    d = dcol.reshape(b, ho, wo, kp)
    for ky in range(3):
        for kx in range(3):
            tap = ky * 3 + kx
            dxp[:, ky:ky + 2 * ho:2, kx:kx + 2 * wo:2, :] += d[..., tap * cin:(tap + 1) * cin]
    return dxp[:, 1:h + 1, 1:w + 1, :]


def forward(params, x, quantize=True):
    """x: [B, 60, 80, 2] (the FP16 input values).  Returns (out [B, 16], cache)."""
    q = bf16 if quantize else (lambda a: np.asarray(a, np.float64))
    p = unpack(params)
    b = x.shape[0]
    a = np.asarray(x, np.float64)
    cache = {"b": b, "col": [], "act": []}
    for l, cfg in enumerate(CONVS):
        col = q(im2col(a, cfg))
        bias = np.asarray(p[2 * l + 1], np.float32).astype(np.float64) if quantize else p[2 * l + 1]
        y = col @ q(p[2 * l]).T + bias
        act = q(np.maximum(y, 0.0))
        cache["col"].append(col)
        cache["act"].append(act)
        a = act.reshape(b, cfg[4], cfg[5], cfg[1])
    gap = q(cache["act"][3].reshape(b, 20, 128).mean(axis=1))
    h1 = q(np.maximum(gap @ q(p[8]).T + p[9], 0.0))
    out = h1 @ q(p[10]).T + p[11]
    cache.update(gap=gap, h1=h1, out=out, p=p, q=q)
    return out, cache


def backward(cache, targets):
    """Mean squared error over the 6 outputs; returns (loss, gradient vector)."""
    q, p, b = cache["q"], cache["p"], cache["b"]
    out = cache["out"]
    e = out[:, :OUT] - np.asarray(targets, np.float64)
    loss = float((e ** 2).mean())
    dout = np.zeros((b, OUT_PAD))
    dout[:, :OUT] = 2.0 * e / (b * OUT)
    g = [None] * 12
    dob = q(dout)
    g[10] = dob.T @ cache["h1"]
    g[11] = dout.sum(axis=0)
    dh = (dob @ q(p[10])) * (cache["h1"] > 0)
    dhb = q(dh)
    g[8] = dhb.T @ cache["gap"]
    g[9] = dh.sum(axis=0)
    dgap = dhb @ q(p[8])
    dact = np.repeat(dgap[:, None, :] / 20.0, 20, axis=1).reshape(b * 20, 128)
    for l in range(3, -1, -1):
        cfg = CONVS[l]
        dy = dact * (cache["act"][l] > 0)
        dyb = q(dy)
        g[2 * l + 1] = dy.sum(axis=0)
        g[2 * l] = dyb.T @ cache["col"][l]
        if l == 0:
            break
        dcol = dyb @ q(p[2 * l])
        dact = col2im(dcol, cfg, b).reshape(-1, cfg[0])
    return loss, pack(g)


def loss_only(params, x, targets, quantize=False):
    out, _ = forward(params, x, quantize)
    return float(((out[:, :OUT] - targets) ** 2).mean())


def init_params(seed=0):
    """He-normal convolution and hidden weights, a small output layer, zero
    biases; padding zero (float32 vector)."""
    rng = np.random.default_rng(seed)
    t = []
    for l, cfg in enumerate(CONVS):
        cin, cout, kp = cfg[0], cfg[1], cfg[6]
        w = np.zeros((cout, kp))
        w[:, :9 * cin] = rng.normal(0.0, np.sqrt(2.0 / (9 * cin)), (cout, 9 * cin))
        t += [w, np.zeros(cout)]
    t += [rng.normal(0.0, np.sqrt(2.0 / 128), (FC1, 128)), np.zeros(FC1)]
    w2 = np.zeros((OUT_PAD, FC1))
    w2[:OUT] = rng.normal(0.0, 0.01, (OUT, FC1))
    t += [w2, np.zeros(OUT_PAD)]
    return pack(t).astype(np.float32)
