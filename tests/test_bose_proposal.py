"""The plain sampler's three-term Bose proposal, restated in numpy with the
same term and Gamma-order selection from one selector uniform as the CUDA
try (iss_gb300/csrc/kernels_sample.cu, prop_bose2 / try_once) and the oracle
replay (oracle/oracle_sampler.c, orc_setup / orc_try): accepted K = (E - m)/T
must follow the Bose-Einstein target (K^2 + 2 m~ K + m~^2/2) e^-K /
(1 - e^-(a + K)) of the reference's momentum samplers
(src/BosonMomentumSampler.cpp, src/MomentumSamplerBase.cpp:45-56), the
radial factor that the one-term proposal reaches with acceptance
(1 - e^-a)/(1 - e^-(a + K)).  CPU only."""
import numpy as np
import pytest
from scipy import integrate, stats


def bose3_draws(mt, a, n, rng):
    """Accepted K from the three-term proposal: term j (rate j) has weights
    e^-(j-1)a (2/j^3, 2 m~/j^2, m~^2/(2j)); the selector is rescaled so that
    term j's Gamma(3), Gamma(2), Gamma(1) thresholds are 1 and 1 + j m~."""
    ea = np.exp(-a)
    W1 = 2.0 + 2.0 * mt + 0.5 * mt * mt
    W12 = W1 + 0.25 * ea * (1.0 + mt) ** 2
    W = W12 + (2.0 / 27.0) * ea * ea * (1.0 + 1.5 * mt) ** 2
    r2 = 4.0 / ea
    qa = -np.expm1(-3.0 * a)
    out, tries = [], 0
    while sum(len(o) for o in out) < n:
        m = 2 * n
        U = rng.random((m, 5))
        sel = U[:, 0] * W
        t2, t3 = sel >= W1, sel >= W12
        s = np.where(t3, (sel - W12) * r2 * (0.84375 * r2), np.where(t2, (sel - W1) * r2, 0.5 * sel))
        nt = np.where(t3, 3.0, np.where(t2, 2.0, 1.0))
        prod = 1.0 - U[:, 1]
        prod = np.where(s < 1.0 + nt * mt, prod * (1.0 - U[:, 2]), prod)
        prod = np.where(s < 1.0, prod * (1.0 - U[:, 3]), prod)
        K = -np.log(prod) / nt
        aq = qa / -np.expm1(-3.0 * (a + K))
        assert aq.max() <= 1.0 + 1e-12
        out.append(K[U[:, 4] < aq])
        tries += m
    got = np.concatenate(out)
    return got[:n], tries / len(got)


def target_cdf(mt, a):
    xs = np.linspace(0.0, 80.0, 80001)
    ys = (xs * xs + 2 * mt * xs + 0.5 * mt * mt) * np.exp(-xs) / -np.expm1(-(a + xs))
    c = integrate.cumulative_trapezoid(ys, xs, initial=0.0)
    c /= c[-1]
    return lambda k: np.interp(k, xs, c)


@pytest.mark.parametrize("mt,a", [(0.93, 0.93),   # pion at T = 0.15 GeV
                                  (0.93, 0.12),   # near condensation (the tables stop at a = 0.1)
                                  (3.3, 3.3),     # kaon
                                  (5.2, 1.0),     # heavy meson with a chemical potential
                                  (20.0, 20.0)])  # heavy: the e^-2K, e^-3K terms vanish
def test_three_term_bose_proposal_is_exact(mt, a):
    rng = np.random.default_rng(int(100 * mt + a))
    K, tries = bose3_draws(mt, a, 400_000, rng)
    p = stats.kstest(K, target_cdf(mt, a)).pvalue
    assert p > 1e-3, (mt, a, p)
    # the acceptance of the statistics factor alone: (1 - e^-3a) times the
    # series' mass over its first three terms, at least 1 - e^-3a
    assert 1.0 <= tries <= 1.0 / -np.expm1(-3.0 * a) + 0.01


def test_three_terms_beat_one_for_pions():
    """The statistics factor's acceptance for a pion-like boson: one term
    (1 - e^-a) sum_n I_n / I_1 against three terms, I_n the n-th term's mass."""
    mt = a = 0.93
    n = np.arange(1, 200)
    In = np.exp(-n * a) * (2.0 / n ** 3 + 2.0 * mt / n ** 2 + mt * mt / (2.0 * n))
    acc1 = -np.expm1(-a) * In.sum() / In[0]
    acc3 = -np.expm1(-3 * a) * In.sum() / In[:3].sum()
    assert acc1 == pytest.approx(0.669, abs=0.005)
    assert acc3 == pytest.approx(0.943, abs=0.005)
