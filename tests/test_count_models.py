"""The count models other than Poisson (dN_dy_sampling_model 1, 10, 20) and
the event count of sample_upto_desired_particle_number = 1, on the GPU
against the oracle.

* determine_number_to_sample (src/FSSW.cpp:250-309): model 1 is the integer
  part plus a Bernoulli draw of the fractional part, model 10 the integer
  part plus a negative-binomial draw of the fractional part, model 20 a
  negative binomial of the whole yield (Gamma-Poisson mixture, shape
  para1 * mean).  The GPU counts must equal the oracle's replay on the same
  Philox streams bit for bit, and so must the species ids of every hadron.
* compute_number_of_sampling_needed (src/FSSW.cpp:851-869): the number of
  events the generate picks equals the oracle's restatement from its FP64
  yields, and the counts of those events equal the oracle's.
"""
import numpy as np
import pytest

import oracle_lib as O
from iss_gb300 import surfaces as S
from test_gpu_parity import run_golden_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("model,para1", [(1, 0.16), (10, 0.16), (10, 2.0), (20, 0.16), (20, 2.0)])
def test_count_models_match_oracle(model, para1):
    g = O.load_golden("yields_viscous_14moment.npz")
    n_events = 300
    s, params = run_golden_case(g, n_events=n_events, seed=515,
                                extra={"dN_dy_sampling_model": model,
                                       "dN_dy_sampling_para1": para1})
    tot = s.species_yields()
    cnt = s.counts()
    oc = O.OracleConfig(params, S.TABLE_DIR, n_events=n_events, seed=515)
    ref = O.counts(oc, g["species"], tot)
    assert cnt.shape == ref.shape
    assert np.array_equal(cnt, ref), f"{(cnt != ref).sum()} counts differ from the oracle"
    had, off = s.all_hadrons()
    assert len(had) == cnt.sum() > 0
    assert np.array_equal(off[1:] - off[:-1], cnt.sum(1))
    pids = s.species()
    expect = np.concatenate([np.repeat(pids, cnt[e]) for e in range(n_events)])
    assert np.array_equal(had["pid"], expect)
    # the models' own moments for the largest yield: model 1 stays within one
    # of the mean; the reference's negative binomials (gsl_ran_negative_binomial
    # with p = 1/(1 + para1), n = para1 times the fraction or the yield) have
    # mean n para1 and variance n para1 (1 + para1)
    k = int(np.argmax(tot))
    dN = tot[k]
    c = cnt[:, k].astype(np.float64)
    if model == 1:
        assert np.all(np.abs(cnt - tot[None, :]) < 1.0)
    else:
        n_nb = para1 * (dN - np.floor(dN) if model == 10 else dN)
        mean = (np.floor(dN) if model == 10 else 0.0) + n_nb * para1
        var = n_nb * para1 * (1.0 + para1)
        assert abs(c.mean() - mean) < 5.0 * np.sqrt(var / n_events)
        assert 0.4 < c.var() / var < 2.5
    s.close()


def test_sample_upto_desired_particle_number_matches_oracle():
    g = O.load_golden("yields_viscous_14moment.npz")
    extra = {"sample_upto_desired_particle_number": 1, "number_of_particles_needed": 2000,
             "maximum_sampling_events": 5000}
    s, params = run_golden_case(g, n_events=7, seed=88, extra=extra)
    lrf = s.lrf_cells()
    keep = (lrf[:, 4] >= 0).astype(np.int32)
    sp = g["species"]
    oc = O.OracleConfig(params, S.TABLE_DIR, n_events=1, seed=88)
    y64 = O.yields(oc, sp, lrf, keep)
    nev = O.events_needed(params, sp, y64)
    assert 1 < nev < 5000
    assert s.get_number_of_sampled_events() == nev
    cnt = s.counts()
    assert cnt.shape[0] == nev
    oc = O.OracleConfig(params, S.TABLE_DIR, n_events=nev, seed=88)
    assert np.array_equal(cnt, O.counts(oc, sp, s.species_yields()))
    # the cap: maximum_sampling_events bounds it
    s.set_params(maximum_sampling_events=3)
    s.generate_samples()
    assert s.get_number_of_sampled_events() == 3
    s.close()
