"""The streamed generate (iss_gpu_generate_stream): hadrons handed to the
caller chunk by chunk through a device buffer of two chunks.

The concatenated chunks must be the hadrons iss_gpu_generate draws for the
same seed, bit for bit, with the same event offsets, for one surface and
for a batch of surfaces, whatever the chunk size; a second streamed call
must give the same again; afterwards the handle holds no hadrons; decays
are refused."""
import numpy as np
import pytest

from iss_gb300 import iSS, native, surfaces as S

pytestmark = pytest.mark.gpu

PARAMS = dict(S.DEFAULT_PARAMETERS, hydro_mode=2, afterburner_type=0, include_deltaf_shear=1,
              include_deltaf_bulk=1, bulk_deltaf_kind=11, turn_on_bulk=1)


def _collect(s, chunk):
    parts, offs, firsts = [], [], []

    def fn(had, first, off):
        parts.append(had.copy())
        firsts.append(first)
        offs.append(off)

    s.generate_stream(chunk, fn)
    had = np.concatenate(parts) if parts else np.zeros(0, dtype=native.HADRON_DTYPE)
    # global event offsets from the per-chunk ones
    glob = [0]
    for o in offs:
        glob.extend((glob[-1] + o[1:]).tolist())
    return had, np.array(glob, dtype=np.int64), firsts


@pytest.mark.parametrize("chunk", [1, 7, 64, 1000])
def test_stream_equals_generate_single_surface(chunk):
    s = iSS(".", inputfile="")
    s.set_params(**dict(PARAMS, number_of_repeated_sampling=150))
    s.set_surface(S.viscous_3d(5000, seed=4).fo_surf())
    s.set_random_seed(606)
    s.generate_samples()
    ref, ref_off = s.all_hadrons()
    s.set_random_seed(606)
    had, off, firsts = _collect(s, chunk)
    assert firsts == list(range(0, 150, min(chunk, 150)))
    assert np.array_equal(off, ref_off)
    assert had.tobytes() == ref.tobytes()
    with pytest.raises(native.IssError):
        s.all_hadrons()          # a streamed generate keeps no hadrons
    # again, on the same handle
    s.set_random_seed(606)
    had2, _, _ = _collect(s, chunk)
    assert had2.tobytes() == ref.tobytes()
    s.close()


def test_stream_equals_generate_batch():
    surfs = [S.viscous_3d(n, seed=30 + i).fo_surf() for i, n in enumerate((3000, 800, 5000))]
    events = [40, 5, 90]
    s = iSS(".", inputfile="")
    s.set_params(**PARAMS)
    s.set_surface_batch(surfs, events)
    s.set_random_seed(77)
    s.generate_samples()
    ref, ref_off = s.all_hadrons()
    s.set_random_seed(77)
    had, off, _ = _collect(s, 16)
    assert np.array_equal(off, ref_off)
    assert had.tobytes() == ref.tobytes()
    s.close()


def test_stream_refuses_decays():
    s = iSS(".", inputfile="")
    s.set_params(**dict(PARAMS, number_of_repeated_sampling=10, perform_decays=1))
    s.set_surface(S.viscous_3d(500, seed=4).fo_surf())
    s.set_random_seed(1)
    with pytest.raises(native.IssError):
        s.generate_stream(4, lambda *a: None)
    s.close()


@pytest.mark.parametrize("extra", [{"local_charge_conservation": 1},
                                   {"MC_sampling": 2, "bulk_deltaf_kind": 1, "restrict_deltaf": 1,
                                    "deltaf_max_ratio": 1.0, "sample_pT_up_to": -1,
                                    "sample_y_minus_eta_s_range": 3}],
                         ids=["local_charge_conservation", "MC_sampling_2"])
def test_stream_equals_generate_other_samplers(extra):
    """Pairs of records per draw (local charge conservation) and the
    lab-frame sampler stream bit-identically too."""
    s = iSS(".", inputfile="")
    s.set_params(**dict(PARAMS, number_of_repeated_sampling=40, **extra))
    s.set_surface(S.viscous_3d(2000, seed=9).fo_surf())
    s.set_random_seed(313)
    s.generate_samples()
    ref, ref_off = s.all_hadrons()
    s.set_random_seed(313)
    had, off, _ = _collect(s, 6)
    assert len(ref) > 0
    assert np.array_equal(off, ref_off)
    assert had.tobytes() == ref.tobytes()
    s.close()
