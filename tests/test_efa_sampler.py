"""MC_sampling = 2, the reference's lab-frame EmissionFunctionArray sampler
(src/emissionfunction.cpp:3273-3623, 4188-4421), on the GPU.

Its spectra are checked against the reference's own samples in
tests/test_gpu_statistics.py (samples_efa_*).  Here:
* the yields, counts and output slots are those of the FSSW path (the same
  per-cell yields for shear, bulk kind 1 and diffusion): counts and PDG ids
  agree bit for bit with MC_sampling = 4 for a seed;
* every hadron lies inside the proposal's support (pT <= sample_pT_up_to,
  |y - eta_s| <= sample_y_minus_eta_s_range) and on its cell's position;
* run-to-run output is bit-identical; unsupported options are reported.
"""
import numpy as np
import pytest

from iss_gb300 import IssError, iSS, surfaces as S

pytestmark = pytest.mark.gpu

PARAMS = dict(S.DEFAULT_PARAMETERS, hydro_mode=2, afterburner_type=0, include_deltaf_shear=1,
              include_deltaf_bulk=1, bulk_deltaf_kind=1, turn_on_bulk=1,
              number_of_repeated_sampling=200, restrict_deltaf=1, deltaf_max_ratio=1.0,
              sample_pT_up_to=-1, sample_y_minus_eta_s_range=3)


def run(mc, surf, seed=3, **extra):
    s = iSS(".", inputfile="")
    s.set_params(**dict(PARAMS, MC_sampling=mc, **extra))
    s.set_surface(surf.fo_surf())
    s.set_random_seed(seed)
    s.generate_samples()
    had, off = s.all_hadrons()
    return s, had, off


def test_efa_counts_and_ids_match_fssw():
    surf = S.viscous_3d(3000, seed=4)
    s2, h2, off2 = run(2, surf)
    s4, h4, off4 = run(4, surf)
    assert np.array_equal(s2.counts(), s4.counts())
    assert np.array_equal(off2, off4)
    assert np.array_equal(h2["pid"], h4["pid"])
    assert len(h2) > 10000
    t = s2.timings()
    assert t["n_failures"] == 0 and t["n_tries"] > len(h2)


def test_efa_support_and_positions():
    surf = S.viscous_3d(3000, seed=4)
    s, had, _ = run(2, surf, sample_pT_up_to=2.5, sample_y_minus_eta_s_range=1.5)
    pT = np.hypot(had["px"], had["py"]).astype(np.float64)
    assert pT.max() <= 2.5 * (1 + 1e-5)
    E, pz = had["E"].astype(np.float64), had["pz"].astype(np.float64)
    y = 0.5 * np.log((E + pz) / (E - pz))
    eta_s = 0.5 * np.log((had["t"] + had["z"]).astype(np.float64) /
                         (had["t"] - had["z"]).astype(np.float64))
    assert np.abs(y - eta_s).max() <= 1.5 + 1e-3
    # every hadron sits on a cell: (x, y) of the surface's cells
    rec = surf.fo_surf()
    cells = {(float(a), float(b)) for a, b in zip(rec[:, 1], rec[:, 2])}
    assert all((float(a), float(b)) in cells for a, b in zip(had["x"][:5000], had["y"][:5000]))
    # mass shell
    m = had["mass"].astype(np.float64)
    p2 = (had["px"].astype(np.float64) ** 2 + had["py"] ** 2 + pz ** 2)
    assert np.allclose(E ** 2, m ** 2 + p2, rtol=2e-5, atol=1e-5)


def test_efa_run_to_run_identical_and_boost_invariant():
    surf = S.viscous_3d(2000, seed=8)
    _, a, _ = run(2, surf, seed=11)
    _, b, _ = run(2, surf, seed=11)
    assert a.tobytes() == b.tobytes()
    bi = S.ideal_boost_invariant()
    s = iSS(".", inputfile="")
    s.set_params(**dict(PARAMS, MC_sampling=2, hydro_mode=1, include_deltaf_bulk=0,
                        number_of_repeated_sampling=50))
    s.set_surface(bi.fo_surf())
    s.set_random_seed(5)
    s.generate_samples()
    had, _ = s.all_hadrons()
    E, pz = had["E"].astype(np.float64), had["pz"].astype(np.float64)
    y = 0.5 * np.log((E + pz) / (E - pz))
    assert y.min() > -5.0 - 3.0 - 1e-3 and y.max() < 5.0 + 3.0 + 1e-3
    assert abs(np.mean(y)) < 0.1


def test_efa_unsupported_options():
    surf = S.viscous_3d(100, seed=1)
    s = iSS(".", inputfile="")
    s.set_params(**dict(PARAMS, MC_sampling=2, bulk_deltaf_kind=11))
    s.set_surface(surf.fo_surf())
    with pytest.raises(IssError) as e:
        s.generate_samples()
    assert e.value.status == 4
