"""CPU oracle of the learned proposal network (test infrastructure only).

The product never imports this file; tests/ and bench.py use it to check the
GPU network.  It restates, in numpy FP64, the network of
iss_gb300/csrc/mlp.h and the kernels of iss_gb300/csrc/kernels_mlp.cu:

    features (18, zero-padded to 32) -> 4 x [128, ReLU] -> 64 outputs

with the GPU's rounding points: inputs, weights, hidden activations and the
backward operands dZ are rounded to bf16 (round to nearest even) where the
tensor cores read them; sums are exact here (FP32 on the GPU).  The loss is
the mean negative log-likelihood of the mixture

    q(K, n) = sum_k w_k LN(K; mu_k, sigma_k) vMF(n; v_k)

over K = (E - m) / T > 0 and the unit vector n, where w = softmax(logits),
sigma_k = exp(clamp(s_k, -4, 1.5)) and vMF(n; v) = kappa / (4 pi sinh kappa)
exp(v . n) with kappa = |v|.  The network has no counterpart in the
reference (its momentum sampler is src/FSSW.cpp:1852-1966).

`exact=True` switches every bf16 rounding off: that is the pure-FP64 network
whose analytic gradient the finite-difference test checks.
"""
from __future__ import annotations

import numpy as np

N_FEAT, K0, HID, OUT, OUT_USED, NCOMP, NLAYER = 18, 32, 128, 64, 48, 8, 5
LOGSIG_MIN, LOGSIG_MAX = -4.0, 1.5
DIM_IN = [K0, HID, HID, HID, HID]
DIM_OUT = [HID, HID, HID, HID, OUT]


def _offsets():
    off, o = [], 0
    for l in range(NLAYER):
        w = o
        o += DIM_OUT[l] * DIM_IN[l]
        b = o
        o += DIM_OUT[l]
        off.append((w, b))
    return off, o


OFFSETS, N_PARAMS = _offsets()


def bf16(x):
    """Round FP32 values to the nearest bf16 (ties to even), returned as FP64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32)).view(np.uint32).astype(np.uint64)
    r = ((a >> 16) & 1) + 0x7FFF
    b = ((a + r) >> 16).astype(np.uint32) << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    Ws, bs = [], []
    for l, (w, b) in enumerate(OFFSETS):
        Ws.append(p[w:w + DIM_OUT[l] * DIM_IN[l]].reshape(DIM_OUT[l], DIM_IN[l]))
        bs.append(p[b:b + DIM_OUT[l]])
    return Ws, bs


def pack(Ws, bs):
    out = np.zeros(N_PARAMS)
    for l, (w, b) in enumerate(OFFSETS):
        out[w:w + Ws[l].size] = Ws[l].ravel()
        out[b:b + bs[l].size] = bs[l]
    return out


def _r(x, exact):
    return np.asarray(x, dtype=np.float64) if exact else bf16(x)


def forward(params, feats, exact=False):
    """Network outputs [n][64] and the cache the backward pass needs."""
    Ws, bs = unpack(params)
    n = feats.shape[0]
    x = np.zeros((n, K0))
    x[:, :N_FEAT] = feats
    h = _r(x, exact)
    acts = [h]
    for l in range(NLAYER):
        bias = np.asarray(bs[l], dtype=np.float64 if exact else np.float32)
        z = h @ _r(Ws[l], exact).T + bias
        if l < NLAYER - 1:
            h = _r(np.maximum(z, 0.0), exact)
            acts.append(h)
        else:
            h = z
    return h, acts


def log_vmf_norm(kap):
    kap = np.asarray(kap, dtype=np.float64)
    small = kap < 1e-3
    ks = np.where(small, 1.0, kap)
    big = -np.log(4 * np.pi) - ks + np.log(2 * ks) - np.log(-np.expm1(-2 * ks))
    return np.where(small, -np.log(4 * np.pi) - kap ** 2 / 6, big)


def langevin_over_kappa(kap):
    kap = np.asarray(kap, dtype=np.float64)
    small = kap < 1e-2
    ks = np.where(small, 1.0, kap)
    big = (1.0 / np.tanh(ks) - 1.0 / ks) / ks
    return np.where(small, 1.0 / 3 - kap ** 2 / 45, big)


def mixture_logpdf(out, target):
    """log q(K, n) per row (density in dK dOmega) and the pieces of its gradient."""
    z = np.asarray(out, dtype=np.float64)
    K = target[:, 0].astype(np.float64)
    nv = target[:, 1:4].astype(np.float64)
    lK = np.log(K)
    logits = z[:, 0:8]
    lse_w = np.logaddexp.reduce(logits, axis=1)
    mu = z[:, 8:16]
    sraw = z[:, 16:24]
    s = np.clip(sraw, LOGSIG_MIN, LOGSIG_MAX)
    is2 = np.exp(-2 * s)
    v = z[:, 24:48].reshape(-1, 8, 3)
    kap = np.sqrt((v ** 2).sum(-1))
    d = lK[:, None] - mu
    lc = (logits - lse_w[:, None] - s - 0.5 * np.log(2 * np.pi) - 0.5 * d * d * is2
          + log_vmf_norm(kap) + (v * nv[:, None, :]).sum(-1))
    L = np.logaddexp.reduce(lc, axis=1)
    return L - lK, dict(lc=lc, L=L, lse_w=lse_w, d=d, is2=is2, sraw=sraw, v=v, kap=kap, nv=nv)


def loss_and_dout(out, target):
    """Mean negative log-likelihood and its gradient with respect to out."""
    n = out.shape[0]
    logq, c = mixture_logpdf(out, target)
    z = np.asarray(out, dtype=np.float64)
    r = np.exp(c["lc"] - c["L"][:, None])
    w = np.exp(z[:, 0:8] - c["lse_w"][:, None])
    g = np.zeros((n, OUT))
    g[:, 0:8] = w - r
    g[:, 8:16] = -r * c["d"] * c["is2"]
    inside = (c["sraw"] > LOGSIG_MIN) & (c["sraw"] < LOGSIG_MAX)
    g[:, 16:24] = np.where(inside, -r * (c["d"] ** 2 * c["is2"] - 1.0), 0.0)
    gk = langevin_over_kappa(c["kap"])
    gv = -r[:, :, None] * (c["nv"][:, None, :] - gk[:, :, None] * c["v"])
    g[:, 24:48] = gv.reshape(n, 24)
    return -logq.mean(), g / n


def loss_grad(params, feats, target, exact=False):
    """Mean loss and its gradient with respect to the flat parameters.

    The GPU computes dout in FP32, rounds it to bf16 for the tensor-core
    operands and sums the bias gradient from the FP32 values; this follows
    those points (dout rounded through FP32 first)."""
    Ws, bs = unpack(params)
    out, acts = forward(params, feats, exact)
    loss, dout = loss_and_dout(out, target)
    dz = dout if exact else np.asarray(dout, dtype=np.float32).astype(np.float64)
    gW, gb = [None] * NLAYER, [None] * NLAYER
    for l in range(NLAYER - 1, -1, -1):
        dzr = _r(dz, exact)
        gW[l] = dzr.T @ acts[l]
        gb[l] = dz.sum(0)
        if l > 0:
            dh = dzr @ _r(Ws[l], exact)
            dz = np.where(acts[l] > 0, dh, 0.0)
            if not exact:
                dz = dz.astype(np.float32).astype(np.float64)
    return loss, pack(gW, gb)


def initial_like(seed=0):
    """Random parameters in the spirit of the library's initialisation (for
    tests that need a generic network): fan-in uniform weights, pads zero."""
    rng = np.random.default_rng(seed)
    Ws, bs = [], []
    for l in range(NLAYER):
        fan = N_FEAT if l == 0 else DIM_IN[l]
        a = np.sqrt(6.0 / fan) * (0.1 if l == NLAYER - 1 else 1.0)
        W = rng.uniform(-a, a, (DIM_OUT[l], DIM_IN[l]))
        if l == 0:
            W[:, N_FEAT:] = 0
        if l == NLAYER - 1:
            W[OUT_USED:] = 0
        b = rng.uniform(-0.1, 0.1, DIM_OUT[l])
        if l == NLAYER - 1:
            b[OUT_USED:] = 0
            b[8:16] = np.log(0.25 * 1.6 ** np.arange(8))
            b[16:24] = np.log(0.5)
        Ws.append(W)
        bs.append(b)
    return pack(Ws, bs).astype(np.float32)


def random_targets(n, seed=0):
    """(K, n_x, n_y, n_z) with K ~ Gamma(3) and isotropic directions."""
    rng = np.random.default_rng(seed)
    K = rng.gamma(3.0, 1.0, n)
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return np.column_stack([K, v]).astype(np.float32)
