"""Launch shape, autotuning and graph replay change the time, never a result.

* Every launch shape (draws per work item, species groups per cell, sampler
  and cell-assignment blocks per SM, copy chunks) gives bit-identical
  hadrons: every random number is keyed by (draw, hadron, event, species).
* The autotuner returns a valid shape, no slower than the default, and the
  results stay bit-identical.
* gpu_graph = 1: graph replays give the eager run's hadrons, counts and
  event offsets bit for bit, for new seeds and event offsets; a new shape
  recaptures; a call that outgrows the captured buffers (same cells, twice
  the hadrons) is detected on the device and rerun eagerly.
"""
import numpy as np
import pytest

from conftest import gpu_available  # noqa: F401
from iss_gb300 import IssError, iSS, surfaces as S

PARAMS = dict(S.DEFAULT_PARAMETERS, hydro_mode=2, afterburner_type=0, include_deltaf_shear=1,
              include_deltaf_bulk=1, bulk_deltaf_kind=11, turn_on_bulk=1, quantum_statistics=1,
              dN_dy_sampling_model=30, number_of_repeated_sampling=50)
DEFAULT = {"item_size": 64, "yield_groups": 4, "sampler_ctas": 3, "assign_blocks": 8,
           "copy_chunks": 16}


def handle(surf, **extra):
    s = iSS(".", inputfile="")
    s.set_params(**dict(PARAMS, **extra))
    s.set_surface(surf.fo_surf())
    return s


def run(s, seed):
    s.set_random_seed(seed)
    s.generate_samples()
    had, off = s.all_hadrons()
    return had.copy(), off.copy(), s.counts()


def test_tuning_defaults_and_validation():
    s = iSS(".", inputfile="")
    assert s.get_tuning() == DEFAULT
    for bad in ({"item_size": 48}, {"item_size": 2048}, {"sampler_ctas": 4},
                {"yield_groups": 0}, {"assign_blocks": 33}, {"copy_chunks": 0}):
        with pytest.raises(IssError):
            s.set_tuning(**bad)
    s.set_tuning(item_size=256, copy_chunks=5)
    assert s.get_tuning()["item_size"] == 256 and s.get_tuning()["copy_chunks"] == 5


@pytest.mark.gpu
def test_launch_shapes_give_identical_hadrons():
    surf = S.viscous_3d(20000, seed=2)
    s = handle(surf)
    ref, ref_off, ref_cnt = run(s, 11)
    shapes = [dict(item_size=32, yield_groups=1, sampler_ctas=2, assign_blocks=4, copy_chunks=3),
              dict(item_size=256, yield_groups=16, sampler_ctas=3, assign_blocks=16, copy_chunks=7),
              dict(item_size=1024, yield_groups=8, sampler_ctas=1, assign_blocks=1, copy_chunks=64)]
    for shape in shapes:
        s.set_tuning(**shape)
        had, off, cnt = run(s, 11)
        assert np.array_equal(cnt, ref_cnt), shape
        assert np.array_equal(off, ref_off), shape
        assert had.tobytes() == ref.tobytes(), shape
        # generate_into with the shape's copy chunks
        out = np.zeros(len(ref) + 1000, dtype=ref.dtype)
        s.set_random_seed(11)
        h2, off2 = s.generate_into(out)
        assert h2.tobytes() == ref.tobytes() and np.array_equal(off2, ref_off), shape


@pytest.mark.gpu
def test_autotune_keeps_results():
    surf = S.viscous_3d(50000, seed=2)
    s = handle(surf)
    ref, _, _ = run(s, 5)
    shape, before, after = s.autotune()
    print("autotune:", shape, f"{before:.3f} ms -> {after:.3f} ms")
    assert shape["item_size"] % 32 == 0 and 1 <= shape["sampler_ctas"] <= 3
    assert after <= before * 1.10
    had, _, _ = run(s, 5)
    assert had.tobytes() == ref.tobytes()
    # gpu_autotune = 1 on a new handle of the same shape takes the cached shape
    s2 = handle(surf, gpu_autotune=1)
    had2, _, _ = run(s2, 5)
    assert s2.get_tuning() == shape
    assert had2.tobytes() == ref.tobytes()


@pytest.mark.gpu
def test_graph_replay_matches_eager():
    surf = S.viscous_3d(20000, seed=2)
    eager = handle(surf)
    graph = handle(surf, gpu_graph=1)
    for seed, offset in ((1, 0), (2, 0), (3, 50), (4, 0)):
        eager.set_params(gpu_event_offset=offset)
        graph.set_params(gpu_event_offset=offset)
        a = run(eager, seed)
        b = run(graph, seed)
        assert a[0].tobytes() == b[0].tobytes(), seed
        assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2]), seed
        tg = graph.timings()
        assert tg["n_hadrons"] == len(b[0]) and tg["ms_total"] > 0
    # replays launch the captured graph (18 kernels in one launch)
    assert graph.timings()["kernel_launches"] == 18
    # a new shape (more events) is captured anew
    eager.set_params(number_of_repeated_sampling=80)
    graph.set_params(number_of_repeated_sampling=80)
    for seed in (7, 8):
        a, b = run(eager, seed), run(graph, seed)
        assert a[0].tobytes() == b[0].tobytes()
    # the same shape with twice the hadrons: the graph's buffers are too small,
    # the call reruns eagerly and still gives the eager result
    rec = surf.fo_surf().copy()
    rec[:, 4:8] *= 2.0
    eager.set_surface(rec)
    graph.set_surface(rec)
    a, b = run(eager, 9), run(graph, 9)
    assert len(a[0]) > 1.5 * len(run(handle(surf, number_of_repeated_sampling=80), 9)[0])
    assert a[0].tobytes() == b[0].tobytes()
    assert np.array_equal(a[2], b[2])


@pytest.mark.gpu
def test_two_handles_on_two_threads_match_sequential_runs():
    """Two handles driven concurrently from two host threads (each with its
    own output buffer, both calling generate_into in turn, as bench.py's
    e2e leg does) give every step's hadrons bit for bit as one handle
    sampling the same seeds alone."""
    import threading

    import torch
    surf = S.viscous_3d(30000, seed=2)
    seeds = [[21, 23, 25], [22, 24, 26]]
    ref = {}
    solo = handle(surf)
    for sd in sum(seeds, []):
        had, off, _ = run(solo, sd)
        ref[sd] = (had, off)
    cap = max(len(h) for h, _ in ref.values()) + 1000
    handles = [handle(surf), handle(surf)]
    got = {}
    errors = []

    def work(j):
        try:
            torch.cuda.set_device(0)
            out = np.zeros(cap, dtype=ref[21][0].dtype)
            for sd in seeds[j]:
                handles[j].set_random_seed(sd)
                h, off = handles[j].generate_into(out)
                got[sd] = (h.copy(), off.copy())
        except Exception as e:
            errors.append(e)

    threads = [threading.Thread(target=work, args=(j,)) for j in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for sd, (had, off) in ref.items():
        assert got[sd][0].tobytes() == had.tobytes(), sd
        assert np.array_equal(got[sd][1], off), sd
