"""CPU restatement (FP64, NumPy) of the learned momentum closure.

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` as the checker of the GPU
network kernels (``pysph_gb300/csrc/mlp.cu``), never by the product path.

The reference PySPH has no learned closure; what this checks is the network
the closure uses in place of the momentum pair loop of
``sph/funcs/pressure_funcs.pyx:40-91`` (SPHPressureGradient) and
``sph/funcs/viscosity_funcs.pyx:41-124`` (MonaghanArtificialVsicosity):

* features: for every destination particle the 32 nearest neighbours within
  ``radius_scale * h_i`` (self included, ordered by squared distance, ties
  by sorted source slot), each as ``((x_i-x_j)/h_i, (y_i-y_j)/h_i,
  (u_j-u_i)/c0, (v_j-v_i)/c0, rho_j, p_j)``, standardised per channel;
  missing neighbours are zero rows;
* network: 192 -> 128 -> 128 -> 2 with GELU in its tanh form
  (Hendrycks & Gimpel 2016), weights and the
  activations that feed a matrix product in BF16 (round to nearest even),
  products accumulated in FP32 on the GPU (FP64 here);
* loss ``0.5 / B * sum (y - t)^2`` and its gradient, with the kernels'
  rounding points: the output gradients of the two hidden layers are
  rounded to BF16 before they multiply ``W2`` and the layer inputs, the
  bias gradients are sums of those rounded values, the third layer is FP32.

``emulate=False`` drops every rounding: then ``backward`` is the exact
gradient of the FP64 loss, which ``finite_difference`` checks.
"""
import numpy as np

NIN, NH, NOUT = 192, 128, 2
NNBR, NCH = 32, 6
OFF_W1 = 0
OFF_B1 = OFF_W1 + NH * NIN
OFF_W2 = OFF_B1 + NH
OFF_B2 = OFF_W2 + NH * NH
OFF_W3 = OFF_B2 + NH
OFF_B3 = OFF_W3 + NOUT * NH
NPARAM = OFF_B3 + NOUT


def bf16(a):
    """Round to BFloat16 (nearest, ties to even) through FP32; FP64 out."""
    f = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (u & 0xFFFFFFFF).astype(np.uint32).view(np.float32).astype(np.float64)


GELU_C = np.sqrt(2.0 / np.pi)


def gelu(z):
    """GELU, tanh form (Hendrycks & Gimpel 2016)."""
    return 0.5 * z * (1.0 + np.tanh(GELU_C * (z + 0.044715 * z ** 3)))


def dgelu(z):
    t = np.tanh(GELU_C * (z + 0.044715 * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * GELU_C * (1.0 + 3 * 0.044715 * z * z)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[OFF_W1:OFF_B1].reshape(NH, NIN), p[OFF_B1:OFF_W2],
            p[OFF_W2:OFF_B2].reshape(NH, NH), p[OFF_B2:OFF_W3],
            p[OFF_W3:OFF_B3].reshape(NOUT, NH), p[OFF_B3:NPARAM])


def pack(W1, b1, W2, b2, W3, b3):
    return np.concatenate([W1.ravel(), b1, W2.ravel(), b2, W3.ravel(), b3])


def forward(params, x, emulate=True):
    """y [B, 2] and the cache of intermediate values."""
    r = bf16 if emulate else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, W3, b3 = unpack(params)
    W1, W2, W3 = r(W1), r(W2), r(W3)
    xb = r(x)
    z1 = xb @ W1.T + b1
    h1 = r(gelu(z1))
    z2 = h1 @ W2.T + b2
    h2 = r(gelu(z2))
    y = h2 @ W3.T + b3
    return y, dict(x=xb, z1=z1, h1=h1, z2=z2, h2=h2, W2=W2, W3=W3)


def backward(params, x, target, emulate=True, inv_count=None):
    """(loss, grad[NPARAM]) of 0.5 * inv_count * sum (y - t)^2."""
    r = bf16 if emulate else (lambda a: np.asarray(a, np.float64))
    y, c = forward(params, x, emulate)
    B = y.shape[0]
    s = 1.0 / B if inv_count is None else inv_count
    e = y - target
    loss = 0.5 * s * float(np.sum(e * e))
    dy = e * s
    dW3 = dy.T @ c["h2"]
    db3 = dy.sum(0)
    dh2 = dy @ c["W3"]
    dz2 = r(dh2 * dgelu(c["z2"]))
    dW2 = dz2.T @ c["h1"]
    db2 = dz2.sum(0)
    dh1 = dz2 @ c["W2"]
    dz1 = r(dh1 * dgelu(c["z1"]))
    dW1 = dz1.T @ c["x"]
    db1 = dz1.sum(0)
    return loss, pack(dW1, db1, dW2, db2, dW3, db3)


def finite_difference(params, x, target, idx, eps=1e-6):
    """Central differences of the unrounded FP64 loss at parameters idx."""
    out = []
    for i in idx:
        p = np.array(params, dtype=np.float64)
        p[i] += eps
        lp, _ = backward(p, x, target, emulate=False)
        p[i] -= 2 * eps
        lm, _ = backward(p, x, target, emulate=False)
        out.append((lp - lm) / (2 * eps))
    return np.array(out)


def adam(params, grad, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update (bias-corrected); returns new (params, m, v)."""
    m = beta1 * m + (1 - beta1) * grad
    v = beta2 * v + (1 - beta2) * grad * grad
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    return params - lr * mh / (np.sqrt(vh) + eps), m, v


def init_params(seed=0):
    """Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases."""
    rng = np.random.default_rng(seed)
    W1 = rng.uniform(-1, 1, (NH, NIN)) / np.sqrt(NIN)
    W2 = rng.uniform(-1, 1, (NH, NH)) / np.sqrt(NH)
    W3 = rng.uniform(-1, 1, (NOUT, NH)) / np.sqrt(NH)
    return pack(W1, np.zeros(NH), W2, np.zeros(NH), W3, np.zeros(NOUT))


def features(props, c0, mean, inv_std, radius_scale=2.0):
    """Raw-then-standardised features [N, 192] of a 2D particle set on itself.

    Neighbours: FP64 ``r^2 < (radius_scale h_i)^2`` (base/nnps.pyx:337-353),
    ordered by squared distance then index.
    """
    x, y = props["x"], props["y"]
    u, v = props["u"], props["v"]
    h, rho, p = props["h"], props["rho"], props["p"]
    n = len(x)
    out = np.zeros((n, NNBR * NCH))
    mean = np.asarray(mean, np.float64)
    inv_std = np.asarray(inv_std, np.float64)
    for i in range(n):
        dx = x[i] - x
        dy = y[i] - y
        r2 = dx * dx + dy * dy
        rad = radius_scale * h[i]
        nb = np.nonzero(r2 < rad * rad)[0]
        order = nb[np.lexsort((nb, r2[nb]))][:NNBR]
        raw = np.stack([dx[order] / h[i], dy[order] / h[i], (u[order] - u[i]) / c0,
                        (v[order] - v[i]) / c0, rho[order], p[order]], axis=1)
        out[i, :len(order) * NCH] = ((raw - mean) * inv_std).ravel()
    return out
