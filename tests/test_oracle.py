"""The oracle pinned against the reference (CPU only).

The golden files in tests/golden were produced by the reference compiled from
its own sources (tests/golden/make_golden.py); the oracle must reproduce its
local-rest-frame cells and its per-cell FP64 yields bit for bit."""
import numpy as np
import pytest
import scipy.special as sp

import oracle_lib as O
from iss_gb300 import surfaces as S

CASES = ["ideal_boost_invariant", "viscous_14moment", "viscous_rta", "viscous_boltzmann",
         "viscous_ce_smash", "diffusion_smash"]


@pytest.mark.parametrize("name", CASES)
def test_yields_bit_exact_vs_reference(name):
    g = O.load_golden(f"yields_{name}.npz")
    p = g["params"]
    oc = O.OracleConfig(p, S.TABLE_DIR, n_events=1)
    y = O.yields(oc, g["species"], g["lrf"])
    assert np.array_equal(y, g["yields"]), "oracle yields differ from the reference"


@pytest.mark.parametrize("name", [c for c in CASES if c != "viscous_ce_smash"])
def test_lrf_cells_bit_exact_vs_reference(name):
    g = O.load_golden(f"yields_{name}.npz")
    fo = S.music_to_fo_surf(g["records"], int(g["hydro_mode"]))
    lrf, keep = O.lrf_cells(fo)
    kept = lrf[keep == 1]
    assert np.array_equal(kept.view(np.uint32), g["lrf"].view(np.uint32))


@pytest.mark.parametrize("name", CASES)
def test_species_order_vs_reference(name):
    g = O.load_golden(f"yields_{name}.npz")
    p = g["params"]
    ab = 2 if int(g["eos"]) == 91 else int(p.get("afterburner_type", 0))
    sp_ = O.chosen_species(S.TABLE_DIR, ab, int(p.get("quantum_statistics", 1)))
    assert np.array_equal(sp_, g["species"])


def test_special_function_tables_vs_scipy():
    K = np.zeros(O.SF_LEN * 3)
    E = np.zeros(O.SF_LEN * 9)
    O.lib().orc_sf_tables(1, 1, O._p(K), O._p(E))
    x = 0.5 + 0.05 * np.arange(O.SF_LEN)
    K = K.reshape(-1, 3)
    E = E.reshape(-1, 9)
    for j, n in enumerate((1, 2, 3)):
        ref = sp.kn(n, x)
        m = ref > 1e-300
        assert np.max(np.abs(K[m, j] / ref[m] - 1)) < 1e-13
    for j, n in enumerate([2, 4, 6, 8, 10, 12, 14, 16, 18]):
        ref = sp.expn(n, x)
        m = ref > 1e-300
        assert np.max(np.abs(E[m, j] / ref[m] - 1)) < 1e-13


def test_philox_known_answers():
    """Philox4x32-10 known-answer vectors of the Random123 distribution."""
    import ctypes as C
    code = r"""
#include <stdio.h>
#include "philox.h"
int main(void) {
  uint32_t k1[2] = {0, 0}, c1[4] = {0, 0, 0, 0}, o[4];
  orc_philox4x32_10(c1, k1, o); printf("%08x %08x %08x %08x\n", o[0], o[1], o[2], o[3]);
  uint32_t k2[2] = {0xffffffffu, 0xffffffffu}, c2[4] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu};
  orc_philox4x32_10(c2, k2, o); printf("%08x %08x %08x %08x\n", o[0], o[1], o[2], o[3]);
  uint32_t k3[2] = {0xa4093822u, 0x299f31d0u}, c3[4] = {0x243f6a88u, 0x85a308d3u, 0x13198a2eu, 0x03707344u};
  orc_philox4x32_10(c3, k3, o); printf("%08x %08x %08x %08x\n", o[0], o[1], o[2], o[3]);
  return 0;
}
"""
    import os
    import subprocess
    import tempfile
    d = tempfile.mkdtemp()
    src = os.path.join(d, "kat.c")
    open(src, "w").write(code)
    subprocess.check_call(["gcc", "-O1", "-I", O.ORACLE_DIR, src, "-o", os.path.join(d, "kat")])
    out = subprocess.check_output([os.path.join(d, "kat")]).decode().split("\n")
    assert out[0] == "6627e8d5 e169c58d bc57ac4c 9b00dbd8"
    assert out[1] == "408f276d 41c83b0e a20bc7c6 6d5451fd"
    assert out[2] == "d16cfe09 94fdcceb 5001e420 24126ea1"


def test_oracle_counts_are_poisson():
    """Counts drawn on the Philox streams follow Poisson(mean) for small and
    large means (inversion and PTRS branches)."""
    sp_ = O.chosen_species(S.TABLE_DIR, 0)[:4]
    totals = np.array([0.7, 5.0, 40.0, 900.0])
    params = dict(S.DEFAULT_PARAMETERS, hydro_mode=2)
    oc = O.OracleConfig(params, S.TABLE_DIR, n_events=20000, seed=99)
    c = O.counts(oc, sp_, totals)
    for k, mu in enumerate(totals):
        m, v = c[:, k].mean(), c[:, k].var()
        se = np.sqrt(mu / c.shape[0])
        assert abs(m - mu) < 5 * se
        assert abs(v / mu - 1) < 0.1


def test_fixed_point_cdf_properties():
    """orc_cdf: integer rows below 2^62, totals equal to the FP64 sums to
    truncation, edge values (zero rows, -0, NaN, inf, denormals, wide range)."""
    rng = np.random.default_rng(3)
    n = 5000
    rows = [rng.exponential(1.0, n),
            np.zeros(n),
            np.concatenate([[1e30], rng.exponential(1e-20, n - 1)]),
            np.full(n, 1e-42),                                   # denormal
            rng.exponential(1.0, n) * (rng.random(n) < 0.01)]    # mostly zero
    y = np.array(rows, dtype=np.float32)
    y[0, 10] = -0.0
    y[0, 11] = np.nan
    y[0, 12] = -3.0
    cdf, tot = O.cdf(y)
    assert cdf.dtype == np.uint64 and cdf.shape == (5, n + 1)
    assert np.all(cdf[:, 0] == 0)
    assert np.all(np.diff(cdf.astype(object), axis=1) >= 0)
    assert all(int(q) < 2 ** 62 for q in cdf[:, -1])
    clean = np.where(np.isfinite(y) & (y > 0), y, 0).astype(np.float64)
    ref = clean.sum(1)
    for k in range(5):
        if ref[k] == 0:
            assert tot[k] == 0 and cdf[k, -1] == 0
        else:
            # each q loses < 1 unit of 2^-E; the largest yield keeps 62 - L bits
            assert abs(tot[k] - ref[k]) <= 1e-9 * ref[k] + n * 1e-42, (k, tot[k], ref[k])
    # inf is clamped to FLT_MAX, so the row stays finite
    yi = np.ones((1, 8), dtype=np.float32)
    yi[0, 3] = np.inf
    ci, ti = O.cdf(yi)
    assert np.isfinite(ti[0]) and int(ci[0, -1]) < 2 ** 62
    # the draw v = floor(r Q / 2^64), cell = largest i with C[i] <= v, never
    # lands on a cell whose q is 0
    C = [int(c) for c in cdf[4]]
    Q = C[-1]
    q = np.diff(np.array(C, dtype=object))
    for r in rng.integers(0, 2 ** 63, size=2000, dtype=np.int64):
        rr = int(r) * 2 + 1
        v = (rr * Q) >> 64
        i = int(np.searchsorted(np.array(C[:-1], dtype=object), v, side="right")) - 1
        assert C[i] <= v < C[i + 1] and q[i] > 0


def test_local_charge_conservation_pairs():
    """local_charge_conservation = 1 (src/FSSW.cpp:931-938, 1035-1048):
    negatively charged species are not drawn, every hadron of a positive
    species is followed by its partner (-pid, same mass, same cell)."""
    g = O.load_golden("yields_viscous_14moment.npz")
    p = dict(g["params"], number_of_repeated_sampling=4, local_charge_conservation=1)
    oc = O.OracleConfig(p, S.TABLE_DIR, n_events=4, seed=9)
    lrf = g["lrf"]
    y = g["yields"].astype(np.float32)
    cdf, tot = O.cdf(y)
    sp_ = g["species"]
    cnt = O.counts(oc, sp_, tot)
    assert np.all(cnt[:, sp_["charge"] < 0] == 0)
    assert np.all(cnt[:, sp_["charge"] > 0] % 2 == 0)
    assert cnt[:, sp_["charge"] > 0].sum() > 0
    coef = O.cell_coeffs(oc, lrf).astype(np.float32)
    had, st = O.sample_replay(oc, sp_, lrf, coef, cdf, cnt)
    assert len(had) == cnt.sum() and st.n_failures == 0
    pos = np.isin(had["pid"], sp_["pid"][sp_["charge"] > 0])
    first = np.flatnonzero(pos)
    # records of positive species come in (hadron, partner) pairs
    seg_start = np.concatenate([[0], np.cumsum(cnt.ravel())])[:-1]
    pairs = []
    for e in range(cnt.shape[0]):
        for k in np.flatnonzero(sp_["charge"] > 0):
            b = seg_start[e * len(sp_) + k]
            for i in range(cnt[e, k] // 2):
                pairs.append((b + 2 * i, b + 2 * i + 1))
    a, b = np.array(pairs).T
    assert np.array_equal(had["pid"][b], -had["pid"][a])
    assert np.array_equal(had["mass"][b], had["mass"][a])
    for f in ("x", "y", "t", "z"):
        assert np.array_equal(had[f][b], had[f][a])
    assert len(first) >= len(pairs)


def test_oracle_replay_respects_counts_and_order():
    g = O.load_golden("yields_viscous_14moment.npz")
    p = dict(g["params"], number_of_repeated_sampling=3)
    oc = O.OracleConfig(p, S.TABLE_DIR, n_events=3, seed=5)
    lrf = g["lrf"]
    y = g["yields"].astype(np.float32)
    cdf, tot = O.cdf(y)
    cnt = O.counts(oc, g["species"], tot)
    coef = O.cell_coeffs(oc, lrf).astype(np.float32)
    had, st = O.sample_replay(oc, g["species"], lrf, coef, cdf, cnt)
    assert len(had) == cnt.sum()
    assert st.n_failures == 0
    # species in mass order inside each event
    pids = g["species"]["pid"]
    expected = np.concatenate([np.repeat(pids, cnt[e]) for e in range(3)])
    assert np.array_equal(had["pid"], expected)
    # on-shell
    m2 = had["E"].astype(float) ** 2 - (had["px"].astype(float) ** 2 + had["py"] ** 2 + had["pz"] ** 2)
    assert np.allclose(np.sqrt(np.maximum(m2, 0)), had["mass"], rtol=1e-3, atol=1e-3)


def test_reference_algorithm_port_matches_reference_samples():
    """Oracle part 3 (the reference's sampling algorithm in C) against
    hadrons sampled by the reference binary: same spectra and multiplicities
    (two-sample chi-square, Bonferroni at 0.01)."""
    from scipy import stats
    g = O.load_golden("samples_static_viscous.npz")
    fo = S.music_to_fo_surf(g["records"], int(g["hydro_mode"]))
    lrf, keep = O.lrf_cells(fo)
    p = dict(S.DEFAULT_PARAMETERS, **g["params"])
    n_ev = 8000
    oc = O.OracleConfig(p, S.TABLE_DIR, n_events=n_ev)
    sp_ = O.chosen_species(S.TABLE_DIR, 0)
    had, n, sec = O.reference_sampler(oc, sp_, lrf, keep, seed=3, capacity=2_000_000)
    assert n == len(had) > 0
    pvals = []
    for pid in (211, 321, 2212, -2212):
        h = had[had["pid"] == pid]
        pT = np.hypot(h["px"].astype(float), h["py"].astype(float))
        a = np.histogram(pT, g["pt_edges"])[0].astype(float)
        b = g[f"pt_{pid}"].astype(float)
        m = (a + b) >= 10
        k1, k2 = np.sqrt(b[m].sum() / a[m].sum()), np.sqrt(a[m].sum() / b[m].sum())
        chi2 = np.sum((k1 * a[m] - k2 * b[m]) ** 2 / (a[m] + b[m]))
        pvals.append(stats.chi2.sf(chi2, m.sum() - 1))
        ma, mb = len(h) / n_ev, g[f"n_{pid}"].mean()
        z = (ma - mb) / np.sqrt(ma / n_ev + mb / int(g["n_events"]))
        pvals.append(2 * stats.norm.sf(abs(z)))
    assert min(pvals) > 0.01 / len(pvals), pvals


@pytest.mark.parametrize("name,n_ev", [("static_viscous", 8000), ("viscous_14moment", 20000)])
def test_gpu_algorithm_replay_matches_reference_samples(name, n_ev):
    """The GPU algorithm (flux-exact directions, Gamma-mixture |p|, one
    combined acceptance), replayed in FP64 on the CPU, against hadrons sampled
    by the reference binary: pT, rapidity and multiplicities per species
    (two-sample chi-square, Bonferroni at 0.01)."""
    from scipy import stats
    g = O.load_golden(f"samples_{name}.npz")
    fo = S.music_to_fo_surf(g["records"], int(g["hydro_mode"]))
    lrf, keep = O.lrf_cells(fo)
    p = dict(S.DEFAULT_PARAMETERS, **g["params"])
    oc = O.OracleConfig(p, S.TABLE_DIR, n_events=n_ev, seed=8, compat_fermion=1)
    sp_ = O.chosen_species(S.TABLE_DIR, 0)
    y = O.yields(oc, sp_, lrf, keep).astype(np.float32)
    cdf, tot = O.cdf(y)
    cnt = O.counts(oc, sp_, tot)
    coef = O.cell_coeffs(oc, lrf).astype(np.float32)
    had, st = O.sample_replay(oc, sp_, lrf, coef, cdf, cnt)
    assert st.n_failures == 0 and st.n_bound_violations == 0
    pvals = []
    for pid in (211, 321, 2212, -2212):
        h = had[had["pid"] == pid]
        E, pz = h["E"].astype(float), h["pz"].astype(float)
        obs = {"pt": np.hypot(h["px"].astype(float), h["py"].astype(float)),
               "y": 0.5 * np.log((E + pz) / (E - pz))}
        for key, edges in (("pt", g["pt_edges"]), ("y", g["y_edges"])):
            a = np.histogram(obs[key], edges)[0].astype(float)
            b = g[f"{key}_{pid}"].astype(float)
            m = (a + b) >= 10
            k1, k2 = np.sqrt(b[m].sum() / a[m].sum()), np.sqrt(a[m].sum() / b[m].sum())
            chi2 = np.sum((k1 * a[m] - k2 * b[m]) ** 2 / (a[m] + b[m]))
            pvals.append(stats.chi2.sf(chi2, m.sum() - 1))
        ma, mb = len(h) / n_ev, g[f"n_{pid}"].mean()
        z = (ma - mb) / np.sqrt(ma / n_ev + mb / int(g["n_events"]))
        pvals.append(2 * stats.norm.sf(abs(z)))
    assert min(pvals) > 0.01 / len(pvals), pvals


def test_decay_replay_conserves_energy_and_ends_stable():
    """The oracle's restatement of the resonance decays (oracle_decay.c):
    every final hadron is stable under the strong interaction, two- and
    three-body decays conserve each event's energy (pole masses), and each
    event's stable primaries appear unchanged and in order in its list
    (src/FSSW.cpp:1746-1779)."""
    dp, dc = O.decay_table(S.TABLE_DIR, 0)
    assert len(dp) == 320 and sum(p.stable for p in dp) == 24
    first = {}
    for i in range(len(dp)):
        first.setdefault(dp[i].pid, i)
    pids = [113, 223, 2214, 3124, 313, -2214, 221, 331, 211, 2212, -211, 111]
    rng = np.random.default_rng(3)
    rows, off = [], [0]
    for e in range(60):
        for _ in range(40):
            pid = int(rng.choice(pids))
            m = dp[first[pid]].mass
            p = rng.normal(0.0, 0.5, 3)
            rows.append((pid, m, np.sqrt(m * m + (p ** 2).sum()), p[0], p[1], p[2], 1.0, 0.0, 0.0, 0.0))
        off.append(len(rows))
    had = np.array(rows, dtype=O.HADRON_DTYPE)
    out, roff, fails = O.decay_replay((dp, dc), 5, np.array(off), had)
    assert fails == 0 and roff[-1] == len(out) > len(had)
    stable = {dp[i].pid for i in range(len(dp)) if dp[i].stable}
    assert set(np.unique(out["pid"]).tolist()) <= stable
    e_in = np.add.reduceat(had["E"].astype(np.float64), np.array(off[:-1]))
    e_out = np.add.reduceat(out["E"].astype(np.float64), roff[:-1])
    assert np.max(np.abs(e_out - e_in) / e_in) < 1e-6
    for e in range(60):
        prim = had[off[e]:off[e + 1]]
        keep = [r.tobytes() for r in prim[np.isin(prim["pid"], list(stable))]]
        j = 0
        for r in out[roff[e]:roff[e + 1]]:
            if j < len(keep) and r.tobytes() == keep[j]:
                j += 1
        assert j == len(keep)
    # the same seed gives the same lists; another seed other decays
    out2, _, _ = O.decay_replay((dp, dc), 5, np.array(off), had)
    assert out2.tobytes() == out.tobytes()
    out3, _, _ = O.decay_replay((dp, dc), 6, np.array(off), had)
    assert out3.tobytes() != out.tobytes()
