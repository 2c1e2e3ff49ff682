"""CPU restatement of the radiance-cache network (numpy). Test infrastructure: only tests,
smoke() and bench.py's CPU legs use it, as the checker of the CUDA kernels.

The reference has no learned component; this network is the cache that terminates
medium paths after a few scattering events. Its definition, shared with the CUDA kernels
(narvalengine_gb300/csrc/mlp.cu), is:

* Query: a scattering vertex in a grid medium, position p in the medium's object space
  (the unit box [-0.5, 0.5]^3, GridMedia.cpp:25-43 maps it to grid coordinates) and the
  incoming ray direction w (world space, unit length).
* Encoding (96 features, BF16): u = p + 0.5 in [0, 1]^3; for each of u.x, u.y, u.z and
  k = 0..11: sin(2^k pi u), cos(2^k pi u) (72 features); for the direction
  a = acos(clamp(w.y, -1, 1)) / pi and b = atan2(w.z, w.x) / (2 pi) + 0.5, k = 0..3:
  sin(2^k pi a), cos(2^k pi a), sin(2^k pi b), cos(2^k pi b) (16 features); 8 zeros.
  Feature order: for each scalar, for each k, (sin, cos). Band k + 1 is computed from band k
  by angle doubling (sin 2x = 2 sin x cos x, cos 2x = cos^2 x - sin^2 x, FP32); only band 0
  calls sin and cos. The doubling amplifies the rounding of band 0 by up to 2^11 at the last
  position band (about 1e-4), below the BF16 rounding of the features (4e-3 relative).
* Network: 96 -> 64 -> 64 -> 64 -> 64 (ReLU after each) -> 16, output rows 0..2 are RGB
  radiance (rows 3..15 are zero weights and never trained). Weights BF16 in the matrix
  products, FP32 accumulation, FP32 bias added after the product, activations rounded to
  BF16 before the next product.
* Loss: relative L2, mean over samples and the 3 channels of (y - t)^2 / (sg(y)^2 + 0.01)
  (sg: no gradient through the denominator).
* Optimiser: Adam on FP32 master weights, lr 1e-2, beta1 0.9, beta2 0.99, eps 1e-8, bias
  corrected; the BF16 copies are re-rounded after each step.
"""
from __future__ import annotations

import numpy as np

IN_FEATURES = 96
HIDDEN = 64
OUT_ROWS = 16
N_HIDDEN_LAYERS = 4
POS_BANDS = 12
DIR_BANDS = 4
LR, BETA1, BETA2, ADAM_EPS = 1e-2, 0.9, 0.99, 1e-8
REL_EPS = 0.01

LAYER_SHAPES = [(HIDDEN, IN_FEATURES)] + [(HIDDEN, HIDDEN)] * (N_HIDDEN_LAYERS - 1) + [(OUT_ROWS, HIDDEN)]


def bf16(x: np.ndarray) -> np.ndarray:
    """Rounds FP32 to the nearest BF16 (ties to even), returned as FP32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)
    nan = np.isnan(x)
    if nan.any():
        out = out.copy()
        out[nan] = np.nan
    return out


def encode(pos_ocs: np.ndarray, dirs: np.ndarray) -> np.ndarray:
    """(N, 3) object-space positions and (N, 3) unit directions -> (N, 96) FP32 features
    (before BF16 rounding)."""
    pos_ocs = np.asarray(pos_ocs, np.float32)
    dirs = np.asarray(dirs, np.float32)
    n = len(pos_ocs)
    u = pos_ocs + np.float32(0.5)
    a = np.arccos(np.clip(dirs[:, 1], -1, 1)) / np.pi
    b = np.arctan2(dirs[:, 2], dirs[:, 0]) / (2 * np.pi) + 0.5
    f = np.zeros((n, IN_FEATURES), np.float32)
    col = 0
    two = np.float32(2.0)
    for v, bands in ((u[:, 0], POS_BANDS), (u[:, 1], POS_BANDS), (u[:, 2], POS_BANDS),
                     (a.astype(np.float32), DIR_BANDS), (b.astype(np.float32), DIR_BANDS)):
        x = (np.float32(np.pi) * v).astype(np.float32)
        sn, cs = np.sin(x).astype(np.float32), np.cos(x).astype(np.float32)
        for k in range(bands):
            f[:, col] = sn
            f[:, col + 1] = cs
            col += 2
            # angle doubling: sin 2x = 2 sin x cos x, cos 2x = cos^2 x - sin^2 x (FP32, this order)
            sn, cs = (two * sn * cs).astype(np.float32), (cs * cs - sn * sn).astype(np.float32)
    assert col == 88
    return f


def init_params(seed: int) -> dict:
    """He-uniform weights (bound sqrt(6 / fan_in)), zero biases, output rows 3..15 zero."""
    rng = np.random.default_rng(seed)
    W, b = [], []
    for i, (o, k) in enumerate(LAYER_SHAPES):
        w = rng.uniform(-1, 1, size=(o, k)).astype(np.float32) * np.float32(np.sqrt(6.0 / k))
        if i == len(LAYER_SHAPES) - 1:
            w[3:] = 0
        if i == 0:
            w[:, 88:] = 0
        W.append(w)
        b.append(np.zeros(o, np.float32))
    return {"W": W, "b": b}


def _q(x, quant):
    return bf16(x) if quant else np.asarray(x, np.float64)


def forward(params: dict, feats: np.ndarray, quant: bool = True):
    """Returns (output (N, 16), list of layer inputs, list of pre-activations). quant=False
    computes in FP64 without BF16 rounding (for finite-difference checks)."""
    x = _q(feats, quant)
    xs, zs = [], []
    n_layers = len(params["W"])
    for i in range(n_layers):
        xs.append(x)
        z = x @ _q(params["W"][i], quant).T + params["b"][i]
        zs.append(z.astype(np.float32) if quant else z)
        if i < n_layers - 1:
            x = _q(np.maximum(z, 0), quant)
    return zs[-1], xs, zs


def loss_and_grad_out(out: np.ndarray, target: np.ndarray, den_from=None):
    """Relative L2 loss over the 3 RGB channels and d loss / d output (N, 16). The
    denominator uses `den_from` (default: the output itself) and carries no gradient."""
    y = out[:, :3].astype(np.float64)
    t = np.asarray(target, np.float64)
    yd = y if den_from is None else np.asarray(den_from, np.float64)[:, :3]
    den = yd * yd + REL_EPS
    n = len(y) * 3
    loss = float(np.sum((y - t) ** 2 / den) / n)
    g = np.zeros(out.shape, dtype=out.dtype)
    g[:, :3] = 2.0 * (y - t) / den / n
    return loss, g


def backward(params: dict, xs, zs, g_out: np.ndarray, quant: bool = True):
    """Gradients of every weight and bias. The error signal is rounded to BF16 before each
    product (as the tensor-core kernels do); weight gradients accumulate in FP32. Bias
    gradients are sums of the same BF16 error signal (the kernel takes them as one more row of
    the weight-gradient product, against an input of ones)."""
    n_layers = len(params["W"])
    gW = [None] * n_layers
    gb = [None] * n_layers
    dt = np.float32 if quant else np.float64
    g = g_out.astype(dt)
    for i in range(n_layers - 1, -1, -1):
        gq = _q(g, quant)
        gW[i] = (gq.T @ xs[i]).astype(dt)
        gb[i] = gq.sum(0).astype(dt)
        if i > 0:
            gx = gq @ _q(params["W"][i], quant)
            g = (gx * (xs[i] > 0)).astype(dt)  # xs[i] = relu(z[i-1]) after rounding
    gW[-1][3:] = 0
    gb[-1][3:] = 0
    gW[0][:, 88:] = 0
    return gW, gb


class Adam:
    def __init__(self, params: dict):
        self.t = 0
        self.m = [np.zeros_like(w) for w in params["W"]] + [np.zeros_like(b) for b in params["b"]]
        self.v = [np.zeros_like(w) for w in params["W"]] + [np.zeros_like(b) for b in params["b"]]

    def step(self, params: dict, gW, gb, lr: float = LR):
        self.t += 1
        ps = params["W"] + params["b"]
        gs = list(gW) + list(gb)
        c1 = 1 - BETA1 ** self.t
        c2 = 1 - BETA2 ** self.t
        for i, (p, g) in enumerate(zip(ps, gs)):
            self.m[i] = BETA1 * self.m[i] + (1 - BETA1) * g
            self.v[i] = BETA2 * self.v[i] + (1 - BETA2) * g * g
            mh = self.m[i] / c1
            vh = self.v[i] / c2
            p -= (lr * mh / (np.sqrt(vh) + ADAM_EPS)).astype(np.float32)


def train_step(params: dict, adam: Adam, feats: np.ndarray, target: np.ndarray) -> float:
    out, xs, zs = forward(params, feats)
    loss, g = loss_and_grad_out(out, target)
    gW, gb = backward(params, xs, zs, g)
    adam.step(params, gW, gb)
    return loss


def predict(params: dict, feats: np.ndarray) -> np.ndarray:
    out, _, _ = forward(params, feats)
    return np.maximum(out[:, :3], 0)
