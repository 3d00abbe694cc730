"""TEST INFRASTRUCTURE: CPU restatement of the radiance-cache MLP.

The reference has no learned component; the radiance cache is an extension
that stands in for its final gather (PhotonMap::radiance_est behind the
diffuse rays of shade_phong, src/shader.cc:154-187, src/pmap.cc:143-178).
This module is the checker of the GPU kernels in sray_gb300/csrc/nrc.cu: the
same encoding, the same network, the same loss and the same Adam update,
written with numpy.  `bf16=True` rounds weights and layer inputs to bfloat16
the way the tensor-core kernels consume them; `bf16=False` is the exact
(float64) function, used to check the backward pass by finite differences.

Network (parameter order of the packed vector, as the C-ABI exchanges it):
  input   9 scalars: position scaled to [0,1]^3, unit normal, unit direction
  encode  for each scalar v and band b = 0..11: sin(pi 2^b v), cos(pi 2^b v)
          -> 216 features, feature index (v * 12 + b) * 2 + (0 sin, 1 cos)
  W1 64x216, b1 64, W2 64x64, b2 64, W3 64x64, b3 64, W4 64x64, b4 64,
  W5 3x64, b5 3           (ReLU after layers 1-4, linear output)
  loss    mean over samples and channels of (y - t)^2 / (sg(y)^2 + 0.01)
  Adam    lr 1e-3, beta1 0.9, beta2 0.999, eps 1e-8
"""
import numpy as np

BANDS = 12
N_IN = 9
N_FEAT = N_IN * BANDS * 2
HID = 64
N_OUT = 3
SHAPES = [(HID, N_FEAT), (HID,), (HID, HID), (HID,), (HID, HID), (HID,), (HID, HID), (HID,), (N_OUT, HID), (N_OUT,)]
N_PARAMS = sum(int(np.prod(s)) for s in SHAPES)
LOSS_EPS = 0.01
LR, BETA1, BETA2, ADAM_EPS = 1e-3, 0.9, 0.999, 1e-8


def bf16(x):
    """Round float32 values to bfloat16 (round to nearest even), as float32."""
    x = np.asarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(x), x, out).astype(np.float32)


def unpack(p):
    out, o = [], 0
    for s in SHAPES:
        n = int(np.prod(s))
        out.append(np.asarray(p[o:o + n], dtype=np.float64).reshape(s))
        o += n
    return out


def pack(ws):
    return np.concatenate([np.asarray(w, dtype=np.float64).ravel() for w in ws])


def init_params(seed):
    """He-uniform weights, zero biases (the GPU side is given these values)."""
    rng = np.random.default_rng(seed)
    ws = []
    for s in SHAPES:
        if len(s) == 2:
            lim = np.sqrt(6.0 / s[1])
            ws.append(rng.uniform(-lim, lim, s))
        else:
            ws.append(np.zeros(s))
    return pack(ws).astype(np.float32)


def encode(x):
    """x: [n, 9] -> [n, 216] float64 features."""
    x = np.asarray(x, dtype=np.float64)
    n = x.shape[0]
    f = np.zeros((n, N_IN, BANDS, 2))
    for b in range(BANDS):
        a = np.pi * (2.0 ** b) * x
        f[:, :, b, 0] = np.sin(a)
        f[:, :, b, 1] = np.cos(a)
    return f.reshape(n, N_FEAT)


def forward(params, x, bf16_ops=True):
    """Returns (outputs [n,3], cache) with the layer inputs and pre-activations."""
    ws = unpack(params)
    rnd = bf16 if bf16_ops else (lambda v: np.asarray(v, dtype=np.float64))
    h = rnd(encode(x)).astype(np.float64)
    hs, zs = [h], []
    for l in range(5):
        W, b = ws[2 * l], ws[2 * l + 1]
        z = h @ rnd(W).astype(np.float64).T + b
        zs.append(z)
        if l < 4:
            h = np.maximum(z, 0.0)
            h = rnd(h).astype(np.float64)
            hs.append(h)
    return zs[-1], (ws, hs, zs)


def loss_and_dy(y, t):
    """Relative L2 and its gradient wrt y (denominator held constant)."""
    y = np.asarray(y, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    den = y * y + LOSS_EPS
    n = y.size
    return float(np.sum((y - t) ** 2 / den) / n), 2.0 * (y - t) / den / n


def backward(cache, dy, bf16_ops=True):
    """Gradients of the loss wrt the packed parameters (float64)."""
    ws, hs, zs = cache
    rnd = bf16 if bf16_ops else (lambda v: np.asarray(v, dtype=np.float64))
    grads = [None] * 10
    dz = np.asarray(dy, dtype=np.float64)
    for l in range(4, -1, -1):
        W = ws[2 * l]
        dzr = rnd(dz).astype(np.float64)
        grads[2 * l] = dzr.T @ hs[l]
        grads[2 * l + 1] = np.sum(dz, axis=0)
        if l > 0:
            dh = dzr @ rnd(W).astype(np.float64)
            dz = dh * (zs[l - 1] > 0)
    return pack(grads)


def adam_step(params, grads, m, v, step):
    """One Adam update (step counts from 1); returns new (params, m, v)."""
    params = np.asarray(params, dtype=np.float64)
    m = BETA1 * m + (1 - BETA1) * grads
    v = BETA2 * v + (1 - BETA2) * grads * grads
    mh = m / (1 - BETA1 ** step)
    vh = v / (1 - BETA2 ** step)
    return params - LR * mh / (np.sqrt(vh) + ADAM_EPS), m, v
