"""Statistical parity of the GPU sampler.

* spectra (pT, y, phi, v2 in pT bins) and mean multiplicities per species
  against hadrons sampled by the reference itself (tests/golden/samples_*),
  for the FSSW sampler (MC_sampling = 4) and the lab-frame sampler
  (MC_sampling = 2, samples_efa_*),
  with the reference's fermion |p| proposal reproduced
  (gpu_compat_fermion_cdf2 = 1); family-wise level 0.01 (Bonferroni);
* |p| of a static ideal cell against the analytic p^2 f(E) spectrum;
* the reference's CI check: T^{mu nu} and n_B rebuilt from the hadrons of
  one-cell surfaces (tests/golden/ci) match the fluid within 1e-3.
"""
import os
import shutil
import tempfile

import numpy as np
import pytest
from scipy import integrate, stats

import oracle_lib as O
from iss_gb300 import iSS, surfaces as S

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ALPHA = 0.01


def two_sample_chi2(a, b):
    """p-value of the two-sample chi-square test of histograms a, b."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    m = (a + b) >= 10
    if m.sum() < 3:
        return 1.0
    a, b = a[m], b[m]
    Na, Nb = a.sum(), b.sum()
    k1, k2 = np.sqrt(Nb / Na), np.sqrt(Na / Nb)
    chi2 = np.sum((k1 * a - k2 * b) ** 2 / (a + b))
    return float(stats.chi2.sf(chi2, m.sum() - 1))


def gof_chi2(counts, probs):
    counts = np.asarray(counts, float)
    exp = probs * counts.sum()
    m = exp >= 10
    chi2 = np.sum((counts[m] - exp[m]) ** 2 / exp[m])
    return float(stats.chi2.sf(chi2, m.sum() - 1))


def sample_case(name, events, seed, compat=1):
    g = O.load_golden(f"samples_{name}.npz")
    surf = S.Surface(g["records"], hydro_mode=int(g["hydro_mode"]), eos=int(g["eos"]),
                     bulk=int(g["music"][0]), rhob=int(g["music"][1]), diff=int(g["music"][2]))
    params = dict(S.DEFAULT_PARAMETERS)
    params.update(g["params"])
    params["number_of_repeated_sampling"] = events
    params["gpu_compat_fermion_cdf2"] = compat
    s = iSS(".")
    s.set_params(**params)
    s.set_surface(surf.fo_surf())
    s.set_random_seed(seed)
    s.generate_samples()
    return g, s


def observables(h):
    px, py, pz, E = (h[k].astype(np.float64) for k in ("px", "py", "pz", "E"))
    return np.hypot(px, py), 0.5 * np.log((E + pz) / (E - pz)), np.arctan2(py, px)


@pytest.mark.parametrize("name,events", [("static_viscous", 40000), ("viscous_14moment", 100000),
                                         ("ideal_boost_invariant", 1000), ("viscous_lcc", 30000),
                                         ("viscous_decays", 20000),
                                         # MC_sampling = 2, the lab-frame sampler
                                         ("efa_viscous_rta", 40000),
                                         ("efa_ideal_boost_invariant", 1000),
                                         ("efa_viscous_lcc", 30000)])
def test_spectra_match_reference_samples(name, events):
    g, s = sample_case(name, events, seed=4242)
    had, off = s.all_hadrons()
    pvals = {}
    nev_ref = int(g["n_events"])
    nev = s.get_number_of_sampled_events()
    for pid in (211, -211, 111, 321, 2212, -2212, 3122):
        h = had[had["pid"] == pid]
        pT, y, phi = observables(h)
        pvals[f"pt {pid}"] = two_sample_chi2(np.histogram(pT, g["pt_edges"])[0], g[f"pt_{pid}"])
        pvals[f"y {pid}"] = two_sample_chi2(np.histogram(y, g["y_edges"])[0], g[f"y_{pid}"])
        pvals[f"phi {pid}"] = two_sample_chi2(np.histogram(phi, g["phi_edges"])[0], g[f"phi_{pid}"])
        # v2 in pT bins: <cos 2 phi> per bin, z-scores combined in a chi-square
        n_a = np.histogram(pT, g["pt_edges"])[0].astype(float)
        v_a = np.histogram(pT, g["pt_edges"], weights=np.cos(2 * phi))[0]
        n_b = g[f"pt_{pid}"].astype(float)
        v_b = g[f"v2num_{pid}"]
        m = (n_a > 50) & (n_b > 50)
        if m.sum() > 2:
            z = (v_a[m] / n_a[m] - v_b[m] / n_b[m]) / np.sqrt(0.5 / n_a[m] + 0.5 / n_b[m])
            pvals[f"v2 {pid}"] = float(stats.chi2.sf(np.sum(z ** 2), m.sum()))
        # mean multiplicity per event (Poisson)
        ev_of = np.repeat(np.arange(nev), np.diff(off))
        counts = np.bincount(ev_of[had["pid"] == pid], minlength=nev)
        ma, mb = counts.mean(), g[f"n_{pid}"].mean()
        if ma + mb > 0:
            z = (ma - mb) / np.sqrt(max(ma, 1e-9) / nev + max(mb, 1e-9) / nev_ref)
            pvals[f"mult {pid}"] = float(2 * stats.norm.sf(abs(z)))
    worst = min(pvals, key=pvals.get)
    assert pvals[worst] > ALPHA / len(pvals), f"{worst}: p = {pvals[worst]:.2e} ({len(pvals)} tests)"
    # spec bar: the bulk of the individual tests at p > 0.01
    frac_low = np.mean([p < 0.01 for p in pvals.values()])
    assert frac_low <= 0.1, f"{frac_low:.2f} of the tests below p = 0.01: {pvals}"


def _static_cell_surface(T=0.150, da0=400.0):
    """One static ideal cell: u = (1, 0, 0, 0), dsigma = (dsigma_0, 0, 0, 0)."""
    e, P = S._eos_s95(np.array([T]))
    rec = np.zeros((1, 34), dtype=np.float32)
    rec[0, 0] = 10.0
    rec[0, 4] = da0
    rec[0, 8] = 1.0
    rec[0, 12] = e[0] / S.HBARC
    rec[0, 13] = T / S.HBARC
    rec[0, 17] = (e[0] + P[0]) / T
    return S.Surface(rec, hydro_mode=2)


def _run_static(events, compat):
    surf = _static_cell_surface()
    s = iSS(".")
    s.set_params(**dict(S.DEFAULT_PARAMETERS, hydro_mode=2, include_deltaf_shear=0,
                        number_of_repeated_sampling=events, gpu_compat_fermion_cdf2=compat))
    s.set_surface(surf.fo_surf())
    s.set_random_seed(99)
    s.generate_samples()
    return s.all_hadrons()[0]


def _expected_p(mass, T, sign, edges):
    """Bin probabilities of |p| for the density p^2 f(E) in the rest frame."""
    def dens(p):
        E = np.sqrt(p * p + mass * mass)
        return p * p / (np.exp(E / T) + sign)
    tot = integrate.quad(dens, 0, 40 * T, limit=400)[0]
    return np.array([integrate.quad(dens, a, b, limit=200)[0]
                     for a, b in zip(edges[:-1], edges[1:])]) / tot


def test_momentum_magnitude_matches_analytic_spectrum():
    had = _run_static(events=20000, compat=0)
    edges = np.linspace(0.0, 2.0, 41)
    T = 0.150
    for pid, mass, sign in ((211, 0.13957, -1), (2212, 0.938272, 1), (321, 0.493677, -1)):
        h = had[had["pid"] == pid]
        p = np.sqrt(h["px"].astype(float) ** 2 + h["py"] ** 2 + h["pz"] ** 2)
        assert len(p) > 20000
        pv = gof_chi2(np.histogram(p, edges)[0], _expected_p(mass, T, sign, edges))
        assert pv > 1e-3, f"|p| of {pid} vs p^2 f(E): p = {pv:.2e}"
        # unbinned: Kolmogorov-Smirnov against the analytic CDF of p^2 f(E)
        grid = np.linspace(0.0, 40 * T, 4001)
        cdf = np.concatenate([[0.0], np.cumsum(_expected_p(mass, T, sign, grid))])[:-1]
        cdf = np.append(cdf, 1.0)[: grid.size]
        ks = stats.kstest(p, lambda x: np.interp(x, grid, cdf)).pvalue
        assert ks > 1e-3, f"|p| of {pid}: KS p = {ks:.2e}"
        # isotropy in the rest frame
        cth = h["pz"].astype(float) / np.maximum(p, 1e-12)
        assert stats.kstest(cth, "uniform", args=(-1, 2)).pvalue > 1e-3
        phi = np.arctan2(h["py"], h["px"])
        assert stats.kstest(phi, "uniform", args=(-np.pi, 2 * np.pi)).pvalue > 1e-3


@pytest.mark.parametrize("cell,music,params,extra", [
    ("testViscousOneFluidCell1.dat", "music_input_91", "iSS_parameters_CEdeltaf.dat", {}),
    ("testViscousOneFluidCell2.dat", "music_input_9", "iSS_parameters_CEdeltaf.dat", {}),
    ("testIdealOneFluidCell1.dat", "music_input_91", "iSS_parameters_ideal.dat",
     {"bulk_deltaf_kind": 21}),
    ("testIdealOneFluidCell2.dat", "music_input_9", "iSS_parameters_ideal.dat",
     {"bulk_deltaf_kind": 21}),
])
def test_reference_ci_tmunu_reconstruction(cell, music, params, extra):
    ci = os.path.join(HERE, "golden", "ci")
    work = tempfile.mkdtemp()
    shutil.copy(os.path.join(ci, cell), os.path.join(work, cell))
    shutil.copy(os.path.join(ci, music), os.path.join(work, "music_input"))
    s = iSS(work, inputfile=os.path.join(ci, params), surface_filename=cell)
    s.set_params(number_of_repeated_sampling=1000, **extra)
    s.read_in_FO_surface()
    s.set_random_seed(31)
    s.generate_samples()
    lrf = s.lrf_cells()
    c = lrf[0].astype(np.float64)
    volume = c[4] / c[8]
    u = c[8:12]
    e, P, Pi, nB = c[12], c[14], c[19], c[15]
    TL = np.diag([e, P + Pi, P + Pi, P + Pi])
    TL[1, 1] += c[20]
    TL[1, 2] = TL[2, 1] = c[21]
    TL[1, 3] = TL[3, 1] = c[22]
    TL[2, 2] += c[23]
    TL[2, 3] = TL[3, 2] = c[24]
    TL[3, 3] += -c[20] - c[23]
    L = np.eye(4)
    L[0, 0] = u[0]
    L[0, 1:] = L[1:, 0] = u[1:]
    L[1:, 1:] += np.outer(u[1:], u[1:]) / (1 + u[0])
    Tf = L @ TL @ L.T
    had, _ = s.all_hadrons()
    nev = s.get_number_of_sampled_events()
    p = np.stack([had[k].astype(np.float64) for k in ("E", "px", "py", "pz")])
    Tp = (p[:, None, :] * p[None, :, :] / p[0]).sum(-1) / (nev * volume)
    sp = O.chosen_species(S.TABLE_DIR, 2 if music.endswith("91") else 1)
    uniq, inv = np.unique(had["pid"], return_inverse=True)
    bar = dict(zip(sp["pid"].tolist(), sp["baryon"].tolist()))
    bvals = np.array([bar.get(int(x), 0) for x in uniq])
    nb_p = bvals[inv].sum() / (nev * volume)
    diff = np.concatenate([(Tf - Tp).ravel(), [nB - nb_p]])
    assert np.mean(np.abs(diff)) < 1e-3, f"mean |dT| = {np.mean(np.abs(diff)):.2e}"
