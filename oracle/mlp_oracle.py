"""CPU oracle of the source-term surrogate (test infrastructure only).

The reference has no learned component: this file restates, in numpy, the
surrogate this project adds (umwm_gb300/csrc/surrogate.hpp), so that the GPU
kernels can be checked against it:

  * features(...)        the input row of a wet point (rotated log-spectrum
                         plus forcing), as k_features builds it;
  * forward / backward   the MLP 1344 -> 512 -> 512 -> 1344 (GELU) with the
                         GPU's rounding points: bf16 inputs, weights and
                         hidden activations, f32 accumulation, f32 output,
                         bf16 output gradient and bf16 back-propagated
                         activation gradients, pre-activations kept in bf16;
  * loss                 mean squared error over the first om*pm columns,
                         optionally weighted per bin by energy_weight of
                         its input feature (the GPU's "surrogate_loss_weight").

It is never part of the product path.
"""
import numpy as np
from scipy.special import erf

FPAD = 1344
HID = 512
NEXTRA = 9
EPS = 1e-15
LN_C0, LN_C1 = -15.0, 8.0
TS = 2.0
WL0, WL1, WMIN = -20.7232658, -11.5129255, 0.01  # ln 1e-9, ln 1e-5, floor


def energy_weight(x):
    """Weight of a target bin from its input feature x = (ln(e + EPS) - LN_C0)
    / LN_C1: a ramp in ln e from WL0 (weight WMIN) to WL1 (weight 1)."""
    w = (np.asarray(x, dtype=np.float32) * np.float32(LN_C1) + np.float32(LN_C0) - np.float32(WL0)) / np.float32(WL1 - WL0)
    return np.clip(w, np.float32(WMIN), np.float32(1.0)).astype(np.float32)

OFF_W1 = 0
OFF_B1 = OFF_W1 + HID * FPAD
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + FPAD * HID
NPARAM = OFF_B3 + FPAD


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32).reshape(a.shape)


def bf16_bits(x):
    """uint16 bit patterns of bf16(x)."""
    return (bf16(x).view(np.uint32) >> 16).astype(np.uint16)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def unpack(w):
    w = np.asarray(w, dtype=np.float32)
    return (w[OFF_W1:OFF_B1].reshape(HID, FPAD), w[OFF_B1:OFF_W2], w[OFF_W2:OFF_B2].reshape(HID, HID),
            w[OFF_B2:OFF_W3], w[OFF_W3:OFF_B3].reshape(FPAD, HID), w[OFF_B3:NPARAM])


def pack(W1, b1, W2, b2, W3, b3):
    return np.concatenate([W1.ravel(), b1, W2.ravel(), b2, W3.ravel(), b3]).astype(np.float32)


def _mm(a, b):
    """f32-accumulated product of f32 operands (computed in f64, rounded once)."""
    return (a.astype(np.float64) @ b.astype(np.float64)).astype(np.float32)


def forward(w, X):
    W1, b1, W2, b2, W3, b3 = unpack(w)
    Xb = bf16(X)
    Z1 = _mm(Xb, bf16(W1).T) + b1
    H1 = bf16(gelu(Z1))
    Z2 = _mm(H1, bf16(W2).T) + b2
    H2 = bf16(gelu(Z2))
    Y = _mm(H2, bf16(W3).T) + b3
    return Y, dict(Xb=Xb, Z1=bf16(Z1), H1=H1, Z2=bf16(Z2), H2=H2)


def _weights(X, f0, weighted, dtype):
    W = np.ones(X.shape, dtype=dtype)
    if weighted:
        W[:, :f0] = energy_weight(bf16(X)[:, :f0])
    return W


def loss_and_grad(w, X, T, f0, weighted=False):
    """Loss and gradient (packed like the parameters) of one batch."""
    W1, b1, W2, b2, W3, b3 = unpack(w)
    n = X.shape[0]
    Y, c = forward(w, X)
    d = np.zeros_like(Y)
    d[:, :f0] = Y[:, :f0] - bf16(T)[:, :f0]
    Wt = _weights(X, f0, weighted, np.float32)
    loss = float((Wt.astype(np.float64) * d.astype(np.float64) ** 2).sum() / (n * f0))
    dY = bf16(np.float32(2.0) * (Wt * d) / np.float32(n * f0))
    gW3 = _mm(dY.T, c["H2"])
    gb3 = dY.sum(0, dtype=np.float64).astype(np.float32)
    dZ2 = bf16(_mm(dY, bf16(W3)) * gelu_grad(c["Z2"]))
    gW2 = _mm(dZ2.T, c["H1"])
    gb2 = dZ2.sum(0, dtype=np.float64).astype(np.float32)
    dZ1 = bf16(_mm(dZ2, bf16(W2)) * gelu_grad(c["Z1"]))
    gW1 = _mm(dZ1.T, c["Xb"])
    gb1 = dZ1.sum(0, dtype=np.float64).astype(np.float32)
    return loss, pack(gW1, gb1, gW2, gb2, gW3, gb3)


def loss_and_grad_exact(w, X, T, f0, weighted=False):
    """Same network in float64 without any rounding (for finite differences)."""
    W1, b1, W2, b2, W3, b3 = (a.astype(np.float64) for a in unpack(w))
    X = X.astype(np.float64)
    T = T.astype(np.float64)
    n = X.shape[0]
    Z1 = X @ W1.T + b1
    H1 = gelu(Z1)
    Z2 = H1 @ W2.T + b2
    H2 = gelu(Z2)
    Y = H2 @ W3.T + b3
    d = np.zeros_like(Y)
    d[:, :f0] = Y[:, :f0] - T[:, :f0]
    Wt = _weights(X, f0, weighted, np.float64)
    loss = (Wt * d ** 2).sum() / (n * f0)
    dY = 2.0 * Wt * d / (n * f0)
    gW3 = dY.T @ H2
    dZ2 = (dY @ W3) * gelu_grad(Z2)
    gW2 = dZ2.T @ H1
    dZ1 = (dZ2 @ W2) * gelu_grad(Z1)
    gW1 = dZ1.T @ X
    g = np.concatenate([gW1.ravel(), dZ1.sum(0), gW2.ravel(), dZ2.sum(0), gW3.ravel(), dY.sum(0)])
    return loss, g


def features(e_ipo, wdir, wspd, ustar, depth, dts, uc, vc, rhorat, fice, th, dth):
    """Input rows (n, FPAD) of n points: e_ipo (n, pm, om) like the
    reference's F(om,pm,i) read back, the rest per point."""
    e = np.asarray(e_ipo, dtype=np.float32)
    n, pm, om = e.shape
    f0 = om * pm
    X = np.zeros((n, FPAD), dtype=np.float32)
    s = np.mod(np.floor((wdir - th[0]) / dth + 0.5).astype(np.int64), pm)
    for i in range(n):
        rot = np.roll(e[i], -s[i], axis=0)  # rot[p'] = e[(p'+s) mod pm]
        X[i, :f0] = (np.log(rot.T.ravel() + np.float32(EPS)) - LN_C0) / LN_C1  # index o*pm + p'
    d = wdir - th[s]
    d = d - 2 * np.pi * np.floor(d / (2 * np.pi) + 0.5)
    cs, sn = np.cos(wdir), np.sin(wdir)
    ex = [wspd / 25.0, d / dth, ustar, np.log(depth) / 8.0, np.full(n, dts / 60.0), uc * cs + vc * sn,
          -uc * sn + vc * cs, rhorat * 800.0, fice]
    for k, v in enumerate(ex):
        X[:, f0 + k] = v
    return X, s
