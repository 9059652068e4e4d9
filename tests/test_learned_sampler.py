"""The learned proposal end to end on the GPU.

* Training rows: the features of each sampled hadron's (cell, species) pair
  against a numpy restatement from the rest-frame cells, and its target
  (K, n) against the hadron boosted back into its cell's rest frame.
* Training on the tensor cores lowers the mixture loss, below the plain
  proposal's negative log-likelihood of the same rows.
* Sampling with the learned proposal (gpu_sampler = 1, exact mode): counts
  and species ids bit-identical to the plain sampler's (they do not depend
  on the momentum sampler); no excess-branch ratio above 1 (exact rejection
  by construction); the share of excess-branch proposals equals its
  expectation c / (M + c); spectra (pT, y, phi, v2 in pT bins) of every
  learned species match the plain GPU sampler on 1,000 events: the number
  of histograms with p < 0.01 is what chance allows for n tests of an exact
  sampler (the binomial tail of Bin(n, 0.01) above it is below 1e-3), and
  none is below the family-wise level 0.01 / n.
* The pilot envelope alone (gpu_learned_exact = 0): the network's proposal
  needs fewer proposals per hadron than the same accept step without it.
"""
import numpy as np
import pytest
from scipy import stats

import oracle_lib as O
from iss_gb300 import iSS, surfaces as S

pytestmark = pytest.mark.gpu
ALPHA = 0.01

PARAMS = dict(S.DEFAULT_PARAMETERS, hydro_mode=2, afterburner_type=0, include_deltaf_shear=1,
              include_deltaf_bulk=1, bulk_deltaf_kind=11, turn_on_bulk=1, quantum_statistics=1,
              dN_dy_sampling_model=30)


def bf16(x):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32)).view(np.uint32).astype(np.uint64)
    r = ((a >> 16) & 1) + 0x7FFF
    return (((a + r) >> 16).astype(np.uint32) << 16).view(np.float32)


def features(lrf, sp):
    """The 18 pair features of the library (iss_gpu.h) for cells lrf [n][28]
    (FO_surf_LRF columns) and one species record per row."""
    lrf = lrf.astype(np.float64)
    T = lrf[:, 13]
    m = sp["mass"].astype(np.float32).astype(np.float64)
    mu = np.minimum(m, sp["baryon"] * lrf[:, 16] + sp["strange"] * lrf[:, 17] + sp["charge"] * lrf[:, 18])
    iep = 1.0 / (lrf[:, 12] + lrf[:, 14])
    da = lrf[:, 4:8]
    nrm = np.abs(da[:, 0]) + np.linalg.norm(da[:, 1:], axis=1)
    f = np.zeros((lrf.shape[0], 18))
    f[:, 0] = (T - 0.15) * 50
    f[:, 1] = 0.5 * mu / T
    f[:, 2:7] = lrf[:, 20:25] * iep[:, None] * 10
    f[:, 7] = lrf[:, 19] * iep * 20
    f[:, 9:12] = lrf[:, 25:28] * iep[:, None] * 10
    f[:, 12:16] = da / nrm[:, None]
    f[:, 16] = 0.1 * m / T
    f[:, 17] = sp["sign"]
    return f


def rest_frame_targets(had, lrf_rows, mass):
    """(K, n) of hadrons boosted back into their cells' rest frames."""
    u = lrf_rows[:, 8:12].astype(np.float64)
    E = had["E"].astype(np.float64)
    p = np.stack([had["px"], had["py"], had["pz"]], 1).astype(np.float64)
    udp = (u[:, 1:] * p).sum(1)
    c = E - udp / (u[:, 0] + 1)
    pr = p - c[:, None] * u[:, 1:]
    p2 = (pr ** 2).sum(1)
    K = p2 / (np.sqrt(mass ** 2 + p2) + mass) / lrf_rows[:, 13]
    return K, pr / np.sqrt(p2)[:, None]


@pytest.fixture(scope="module")
def trained():
    surf = S.viscous_3d(6000, seed=5)
    s = iSS(".", inputfile="")
    s.set_params(**dict(PARAMS, number_of_repeated_sampling=10))
    s.set_surface(surf.fo_surf())
    curve = s.learned_train(n_momenta=4_000_000, first_seed=10, n_seeds=4, n_steps=1500,
                            batch=8192, learning_rate=2e-3, init_seed=1)
    return surf, s, curve


def test_training_rows_match_restatement(trained):
    surf, s, _ = trained
    st = s.learned_stats()
    assert st["n_train_rows"] == 4_000_000
    # the first rows are the first hadrons of the seed-10 run
    p = iSS(".", inputfile="")
    p.set_params(**dict(PARAMS, number_of_repeated_sampling=st["train_events_per_seed"]))
    p.set_surface(surf.fo_surf())
    p.set_random_seed(10)
    p.generate_samples()
    had, _ = p.all_hadrons()
    n = min(len(had), 200_000)
    had = had[:n]
    f_gpu, t_gpu = s.learned_rows(0, n)
    lrf = p.lrf_cells()
    key = {(float(a), float(b)): i for i, (a, b) in enumerate(zip(lrf[:, 1], lrf[:, 2]))}
    cell = np.array([key[(float(a), float(b))] for a, b in zip(had["x"], had["y"])])
    sp = O.chosen_species(S.TABLE_DIR, 0)
    idx = {int(q): k for k, q in enumerate(sp["pid"])}
    spr = sp[np.array([idx[int(q)] for q in had["pid"]])]
    f_ref = bf16(features(lrf[cell], spr))
    same = np.isclose(f_gpu, f_ref, rtol=2 ** -7, atol=1e-6)
    assert same.all(), f"{(~same).sum()} feature values differ by more than one bf16 step"
    assert (f_gpu == f_ref).mean() > 0.999
    K, nv = rest_frame_targets(had, lrf[cell], sp["mass"][[idx[int(q)] for q in had["pid"]]])
    assert np.allclose(t_gpu[:, 0], K, rtol=2e-3, atol=1e-5)
    # the direction of a hadron almost at rest in its cell is ill-conditioned:
    # its float32 lab momentum (E up to ~20 GeV at large rapidity) is rounded
    # by ~1e-7 E, i.e. ~1e-7 E / |p_LRF| in the direction, amplified by the
    # boost's cancellation; compare where E / |p_LRF| < 1000
    mass = sp["mass"][[idx[int(q)] for q in had["pid"]]]
    Trow = lrf[cell][:, 13].astype(np.float64)
    p_lrf = Trow * np.sqrt(K * (K + 2.0 * mass / Trow))
    ok = had["E"] / p_lrf < 1000.0
    assert ok.mean() > 0.999, ok.mean()
    assert np.allclose(t_gpu[ok, 1:], nv[ok], atol=2e-3)


def test_trained_network_beats_the_plain_proposal(trained):
    _, s, curve = trained
    assert np.all(np.isfinite(curve))
    first, last = curve[:20].mean(), curve[-50:].mean()
    st = s.learned_stats()
    print("loss: first", first, "last", last, "plain proposal", st["train_nll_plain"],
          "train ms", st["ms_train"])
    assert last < first - 0.05, (first, last)
    # the trained network is closer to the target than the plain proposal:
    # the loss difference is KL(target || plain) - KL(target || network)
    assert last < st["train_nll_plain"], (last, st["train_nll_plain"])
    assert st["ms_train"] > 0


def spectra_pvalues(a, b):
    out = {}
    pa, pb = (np.hypot(h["px"], h["py"]) for h in (a, b))
    ya, yb = (0.5 * np.log((h["E"] + h["pz"]) / (h["E"] - h["pz"])) for h in (a, b))
    fa, fb = (np.arctan2(h["py"], h["px"]) for h in (a, b))
    edges = np.quantile(np.concatenate([pa, pb]), np.linspace(0, 1, 31))
    out["pT_chi2"] = _chi2(np.histogram(pa, edges)[0], np.histogram(pb, edges)[0])
    out["pT_ks"] = stats.ks_2samp(pa, pb).pvalue
    edges = np.linspace(-4.5, 4.5, 31)
    out["y_chi2"] = _chi2(np.histogram(ya, edges)[0], np.histogram(yb, edges)[0])
    edges = np.linspace(-np.pi, np.pi, 25)
    out["phi_chi2"] = _chi2(np.histogram(fa, edges)[0], np.histogram(fb, edges)[0])
    # v2 in pT bins: two-sample z test of the mean cos 2 phi per bin
    zs = []
    for lo, hi in ((0, 0.5), (0.5, 1.0), (1.0, 2.0), (2.0, 4.0)):
        ca = np.cos(2 * fa[(pa >= lo) & (pa < hi)])
        cb = np.cos(2 * fb[(pb >= lo) & (pb < hi)])
        if len(ca) > 100 and len(cb) > 100:
            zs.append((ca.mean() - cb.mean()) / np.sqrt(ca.var() / len(ca) + cb.var() / len(cb)))
    out["v2_chi2"] = float(stats.chi2.sf(np.sum(np.square(zs)), len(zs))) if zs else 1.0
    return out


def _chi2(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    m = (a + b) >= 10
    a, b = a[m], b[m]
    Na, Nb = a.sum(), b.sum()
    chi2 = np.sum((np.sqrt(Nb / Na) * a - np.sqrt(Na / Nb) * b) ** 2 / (a + b))
    return float(stats.chi2.sf(chi2, m.sum() - 1))


def max_below_001(n):
    """The largest number of p-values below 0.01 among n tests of an exact
    sampler (uniform p-values) that is not rejected at the 1e-3 level: the
    smallest k with P(Bin(n, 0.01) > k) < 1e-3."""
    k = 0
    while stats.binom.sf(k, n, 0.01) >= 1e-3:
        k += 1
    return k


def _learned_run(s, alpha, safety=1.1, seed=77, exact=1):
    s.set_params(gpu_sampler=1, gpu_learned_alpha=alpha, gpu_learned_min_hadrons_per_cell=0.5,
                 gpu_learned_pilot=128, gpu_learned_safety=safety, gpu_learned_exact=exact)
    s.set_random_seed(seed)
    s.generate_samples()
    had, _ = s.all_hadrons()
    out = had, s.counts(), s.learned_stats(), s.timings()
    s.set_params(gpu_sampler=0, gpu_learned_exact=1)
    return out


def test_learned_sampler_matches_plain_sampler(trained):
    surf, s, _ = trained
    n_events = 1000
    s.set_params(number_of_repeated_sampling=n_events, gpu_sampler=0)
    s.set_random_seed(77)
    s.generate_samples()
    plain, _ = s.all_hadrons()
    c_plain = s.counts()
    t_plain = s.timings()
    learned, c_learned, st, t_learned = _learned_run(s, 0.8)
    print("learned sampler:", st, "tries/hadron", st["n_tries"] / st["n_hadrons"],
          "ms plain", t_plain["ms_total"], "ms learned", t_learned["ms_total"])
    np.testing.assert_array_equal(c_plain, c_learned)
    np.testing.assert_array_equal(plain["pid"], learned["pid"])
    assert st["n_species"] >= 3 and st["n_hadrons"] > 0
    # exact rejection: no excess-branch ratio above 1
    assert st["n_violations"] == 0, st
    # the excess branch takes its expected share of the proposals (its mass
    # c = 1 - M (1 - alpha) against M: at least a few per cent at alpha = 0.8)
    assert 0.01 * st["n_tries"] < st["n_excess_tries"] < 0.8 * st["n_tries"], st
    assert st["n_excess_hadrons"] < st["n_hadrons"]
    # the bound of an exact envelope certified by a <= 1 alone: no fewer
    # proposals per hadron than the plain proposal (alpha -> 0, M at its cap)
    _, _, st0, _ = _learned_run(s, 1e-4, safety=1e6)
    assert st0["n_hadrons"] == st["n_hadrons"]
    assert st["n_tries"] >= st0["n_tries"], (st, st0)
    sp = O.chosen_species(S.TABLE_DIR, 0)
    tot = s.species_yields() * n_events
    learned_pids = [int(sp["pid"][k]) for k in np.argsort(-tot)[:st["n_species"]]]
    pvals = {}
    for pid in learned_pids:
        a = plain[plain["pid"] == pid]
        b = learned[learned["pid"] == pid]
        if len(a) < 5000:
            continue
        for k, v in spectra_pvalues(a, b).items():
            pvals[(pid, k)] = v
    assert len(pvals) >= 15
    low = sorted(pvals.items(), key=lambda kv: kv[1])
    print("smallest p-values:", low[:4], "of", len(pvals))
    # per histogram: for an exact sampler every p-value is uniform, so about
    # n / 100 of them fall below 0.01 by chance
    assert sum(v < 0.01 for v in pvals.values()) <= max_below_001(len(pvals)), low[:5]
    assert low[0][1] > ALPHA / len(pvals), low[:5]


def test_network_lowers_the_proposals_of_the_mixture_branch(trained):
    """The pilot envelope alone (gpu_learned_exact = 0) against the same
    accept step without the network (alpha -> 0 with a safety factor so large
    that every envelope sits at its cap 1 / (1 - alpha), i.e. the plain
    sampler's acceptance): the network's proposal needs fewer proposals per
    hadron.  Its envelope is an estimate, so a few ratios exceed 1."""
    surf, s, _ = trained
    s.set_params(number_of_repeated_sampling=400, gpu_sampler=0)
    _, c1, st, _ = _learned_run(s, 0.8, exact=0)
    _, c0, st0, _ = _learned_run(s, 1e-4, safety=1e6, exact=0)
    np.testing.assert_array_equal(c1, c0)
    assert st0["n_species"] == st["n_species"] and st0["n_hadrons"] == st["n_hadrons"]
    assert st["n_excess_tries"] == 0 and st0["n_excess_tries"] == 0
    assert st["n_violations"] <= 3e-3 * st["n_tries"], st
    assert st["n_tries"] < 0.97 * st0["n_tries"], (st, st0)


def test_learned_sampler_exact_at_finite_density():
    """The finite-density configuration (mu_B up to 0.4 GeV, baryon diffusion,
    SMASH species): the network retrained on that surface's plain samples,
    then the exact learned sampler against the plain one on the same events --
    counts and ids bit-identical, no violation, and the spectra of the
    learned species consistent (no more tests below p = 0.01 than chance
    allows, none below the family-wise level)."""
    surf = S.finite_density_3d(6000, seed=3)
    s = iSS(".", inputfile="")
    params = dict(S.DEFAULT_PARAMETERS, hydro_mode=2, afterburner_type=2, include_deltaf_shear=1,
                  include_deltaf_bulk=1, bulk_deltaf_kind=11, turn_on_bulk=1,
                  include_deltaf_diffusion=1, turn_on_rhob=1, turn_on_diff=1,
                  quantum_statistics=1, dN_dy_sampling_model=30, number_of_repeated_sampling=10)
    s.set_params(**params)
    s.set_surface(surf.fo_surf())
    curve = s.learned_train(n_momenta=2_000_000, first_seed=10, n_seeds=4, n_steps=800,
                            batch=8192, learning_rate=2e-3, init_seed=1)
    assert np.all(np.isfinite(curve)) and curve[-50:].mean() < curve[:20].mean()
    s.set_params(number_of_repeated_sampling=600, gpu_sampler=0)
    s.set_random_seed(5)
    s.generate_samples()
    plain, _ = s.all_hadrons()
    c_plain = s.counts()
    learned, c_learned, st, _ = _learned_run(s, 0.8, seed=5)
    np.testing.assert_array_equal(c_plain, c_learned)
    np.testing.assert_array_equal(plain["pid"], learned["pid"])
    assert st["n_species"] >= 3 and st["n_violations"] == 0, st
    pids = s.species()[np.argsort(-s.species_yields())][:st["n_species"]]
    pvals = {}
    for pid in pids[:6]:
        a, b = plain[plain["pid"] == pid], learned[learned["pid"] == pid]
        if len(a) < 5000:
            continue
        for k, v in spectra_pvalues(a, b).items():
            pvals[(int(pid), k)] = v
    assert len(pvals) >= 10
    low = sorted(pvals.items(), key=lambda kv: kv[1])
    assert sum(v < 0.01 for v in pvals.values()) <= max_below_001(len(pvals)), low[:5]
    assert low[0][1] > ALPHA / len(pvals), low[:5]
    s.close()
