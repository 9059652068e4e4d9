"""Edge cases of the graph replay, the lab-frame sampler and the learned
proposal: no events, no learned species, one cell, a seed change between
replays, and the error paths that must not touch the device."""
import numpy as np
import pytest

from iss_gb300 import IssError, iSS, surfaces as S

pytestmark = pytest.mark.gpu

BASE = dict(S.DEFAULT_PARAMETERS, hydro_mode=2, afterburner_type=0, include_deltaf_shear=1,
            include_deltaf_bulk=1, bulk_deltaf_kind=1, turn_on_bulk=1, number_of_repeated_sampling=0,
            sample_pT_up_to=-1, sample_y_minus_eta_s_range=3, restrict_deltaf=1, deltaf_max_ratio=1.0)


def handle(surf, **kw):
    s = iSS(".", inputfile="")
    s.set_params(**dict(BASE, **kw))
    s.set_surface(surf.fo_surf())
    return s


@pytest.mark.parametrize("mc,graph", [(4, 0), (4, 1), (2, 0), (2, 1)])
def test_zero_events(mc, graph):
    s = handle(S.viscous_3d(500, seed=1), MC_sampling=mc, gpu_graph=graph)
    for seed in (1, 2):
        s.set_random_seed(seed)
        s.generate_samples()
        assert s.get_number_of_sampled_events() == 0
        had, off = s.all_hadrons()
        assert len(had) == 0 and list(off) == [0]


@pytest.mark.parametrize("mc", [4, 2])
def test_single_cell_surface(mc):
    surf = S.viscous_3d(1, seed=3)
    s = handle(surf, MC_sampling=mc, number_of_repeated_sampling=500)
    s.set_random_seed(4)
    s.generate_samples()
    had, off = s.all_hadrons()
    assert len(had) > 0 and off[-1] == len(had)
    assert np.all(had["x"] == np.float32(surf.fo_surf()[0, 1]))


def test_graph_replays_change_with_the_seed():
    s = handle(S.viscous_3d(2000, seed=1), MC_sampling=4, number_of_repeated_sampling=20,
               gpu_graph=1)
    runs = []
    for seed in (1, 2, 1):
        s.set_random_seed(seed)
        s.generate_samples()
        runs.append(s.all_hadrons()[0].copy())
    assert runs[0].tobytes() == runs[2].tobytes()
    assert runs[0].tobytes() != runs[1].tobytes()


def test_learned_without_learned_species_is_the_plain_sampler():
    surf = S.viscous_3d(2000, seed=1)
    s = handle(surf, MC_sampling=4, number_of_repeated_sampling=20)
    s.set_random_seed(6)
    s.generate_samples()
    plain = s.all_hadrons()[0].copy()
    s.learned_init_weights(1)
    # no species reaches 1e9 hadrons per cell: every species keeps the plain proposal
    s.set_params(gpu_sampler=1, gpu_learned_min_hadrons_per_cell=1e9)
    s.set_random_seed(6)
    s.generate_samples()
    st = s.learned_stats()
    learned = s.all_hadrons()[0]
    assert st["n_species"] == 0 and st["n_pairs"] == 0
    assert np.array_equal(plain["pid"], learned["pid"])
    close = np.isclose(plain["px"], learned["px"], rtol=1e-5, atol=1e-6)
    assert close.mean() > 0.999


def test_learned_errors():
    s = handle(S.viscous_3d(100, seed=1), MC_sampling=4, number_of_repeated_sampling=5,
               gpu_sampler=1)
    with pytest.raises(IssError) as e:
        s.generate_samples()          # no weights yet
    assert e.value.status == 8
    s.set_params(MC_sampling=2)
    s.learned_init_weights(0)
    with pytest.raises(IssError) as e:
        s.generate_samples()          # the learned proposal is an FSSW option
    assert e.value.status == 4
    with pytest.raises(IssError):
        s.learned_set_weights(np.zeros(10, dtype=np.float32))
