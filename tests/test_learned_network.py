"""The learned proposal's network on the tensor cores against its CPU oracle
(oracle/mlp_oracle.py).

* CPU: the oracle's analytic gradient against central finite differences
  (pure FP64 network), and the flat weight layout against the library's.
* GPU: the tcgen05 GEMM tile against exact products of the bf16 inputs; the
  forward pass and the loss gradient of the bf16 network against the oracle
  with the same rounding points.
"""
import os
import sys

import numpy as np
import pytest

from conftest import REPO
from iss_gb300 import iSS, native

sys.path.insert(0, os.path.join(REPO, "oracle"))
import mlp_oracle as M  # noqa: E402


def test_weight_layout_matches_library():
    assert native.lib().iss_gpu_learned_num_weights() == M.N_PARAMS == 62016


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    params = M.initial_like(5).astype(np.float64)
    # larger output weights so every mixture term carries gradient
    w4, _ = M.OFFSETS[4]
    params[w4:w4 + 48 * 128] *= 5.0
    feats = rng.normal(size=(9, M.N_FEAT))
    tg = M.random_targets(9, seed=4).astype(np.float64)
    loss, g = M.loss_grad(params, feats, tg, exact=True)
    assert np.isfinite(loss)
    idx = []
    for l, (w, b) in enumerate(M.OFFSETS):
        n_w = M.DIM_OUT[l] * min(M.DIM_IN[l], M.N_FEAT if l == 0 else M.DIM_IN[l])
        for _ in range(6):
            o = rng.integers(0, M.OUT_USED if l == 4 else M.DIM_OUT[l])
            i = rng.integers(0, M.N_FEAT if l == 0 else M.DIM_IN[l])
            idx.append(w + o * M.DIM_IN[l] + i)
        for _ in range(3):
            idx.append(b + rng.integers(0, M.OUT_USED if l == 4 else M.DIM_OUT[l]))
        assert n_w > 0
    h = 1e-6
    for j in idx:
        p1, p2 = params.copy(), params.copy()
        p1[j] += h
        p2[j] -= h
        fd = (M.loss_grad(p1, feats, tg, exact=True)[0] - M.loss_grad(p2, feats, tg, exact=True)[0]) / (2 * h)
        assert abs(fd - g[j]) <= 1e-6 + 1e-4 * abs(fd), (j, fd, g[j])


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, 1.0 + 2 ** -9, -2.5, 0.0], dtype=np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                      # exactly halfway: ties to the even mantissa
    assert r[3] == 1.0                      # below halfway: down
    assert r[2] == 1.0 + 2 ** -7            # above halfway: up
    assert r[4] == -2.5 and r[5] == 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("n,k", [(128, 128), (64, 128), (32, 32), (256, 64), (128, 16)])
def test_tcgen05_gemm_tile(n, k):
    rng = np.random.default_rng(n * 1000 + k)
    a = M.bf16(rng.normal(size=(128, k))).astype(np.float32)
    b = M.bf16(rng.normal(size=(n, k))).astype(np.float32)
    c = native.mma_selftest(a.view(np.uint32) >> 16, b.view(np.uint32) >> 16)
    ref = a.astype(np.float64) @ b.astype(np.float64).T
    err = np.abs(c - ref).max() / np.abs(ref).max()
    assert err < 1e-5, f"tcgen05 tile {128}x{n}x{k}: max relative error {err:.2e}"


def _handle():
    s = iSS(".", inputfile="")
    return s


@pytest.mark.gpu
def test_forward_matches_oracle():
    rng = np.random.default_rng(11)
    params = M.initial_like(1)
    feats = rng.normal(size=(1000, M.N_FEAT)).astype(np.float32)
    s = _handle()
    s.learned_set_weights(params)
    out = s.learned_forward(feats)
    ref, _ = M.forward(params.astype(np.float64), feats.astype(np.float64))
    err = np.abs(out - ref) / (np.abs(ref) + 0.05)
    # a hidden unit whose FP32 and FP64 pre-activations round to different
    # bf16 values moves the outputs by about one bf16 step
    assert np.quantile(err, 0.99) < 5e-3 and err.max() < 3e-2, (np.quantile(err, 0.99), err.max())
    np.testing.assert_array_equal(out[:, M.OUT_USED:], np.float32(0.0))
    assert np.array_equal(s.learned_get_weights(), params)


@pytest.mark.gpu
def test_loss_gradient_matches_oracle():
    rng = np.random.default_rng(12)
    params = M.initial_like(2)
    w4, _ = M.OFFSETS[4]
    params[w4:w4 + 48 * 128] *= 5.0
    n = 777                                  # six full tiles and a ragged one
    feats = rng.normal(size=(n, M.N_FEAT)).astype(np.float32)
    tg = M.random_targets(n, seed=13)
    s = _handle()
    s.learned_set_weights(params)
    loss, g = s.learned_loss_grad(feats, tg)
    rloss, rg = M.loss_grad(params.astype(np.float64), feats.astype(np.float64), tg.astype(np.float64))
    assert abs(loss - rloss) < 1e-4 * abs(rloss), (loss, rloss)
    for l, (w, b) in enumerate(M.OFFSETS):
        for name, lo, hi in (("W", w, b), ("b", b, b + M.DIM_OUT[l])):
            ref = rg[lo:hi]
            got = g[lo:hi]
            rel = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-30)
            assert rel < 1e-2, f"layer {l} {name}: relative gradient error {rel:.2e}"
    # padded inputs and outputs get no gradient
    W0 = g[:M.OFFSETS[0][1]].reshape(128, 32)
    assert np.all(W0[:, M.N_FEAT:] == 0)
    W4 = g[w4:M.OFFSETS[4][1]].reshape(64, 128)
    assert np.all(W4[M.OUT_USED:] == 0)
