"""iss_gpu_scan_counts_noalloc: the count-to-slot scan with fixed scratch.

The GPU test calls it through the C ABI on the per-(event, species) counts
of a real iss_gpu_generate. It compares its offsets with what the existing
entry points report for the same run:
  * the event offsets of iss_gpu_copy_all;
  * the cumulative sums of iss_gpu_copy_counts.
It makes two calls in a row, and it also scans a synthetic array of several
hundred tiles. The file name puts it last in collection, so it also runs after
every other test has used the device.
"""
import ctypes as C

import numpy as np
import pytest

from iss_gb300 import iSS, native, surfaces as S

ISS_OK = 0
ISS_ERR_INVALID_ARG = 1
ISS_ERR_CAPACITY = 9
MAX_SEGMENTS = 16384 * 4096


def _fn():
    f = native.lib().iss_gpu_scan_counts_noalloc
    f.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def test_rejects_oversize_and_bad_arguments_before_device_work():
    f = _fn()
    fake = C.c_void_p(256)   # never dereferenced: every case returns before any device work
    assert f(fake, MAX_SEGMENTS + 1, fake, None) == ISS_ERR_CAPACITY
    assert f(fake, 1 << 40, fake, None) == ISS_ERR_CAPACITY
    assert f(fake, -1, fake, None) == ISS_ERR_INVALID_ARG
    assert f(fake, 10, None, None) == ISS_ERR_INVALID_ARG
    assert f(None, 10, fake, None) == ISS_ERR_INVALID_ARG


def _scan_twice(counts_np):
    import torch
    f = _fn()
    n = counts_np.size
    d_counts = torch.from_numpy(np.ascontiguousarray(counts_np, dtype=np.int32)).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    outs = []
    for _ in range(2):
        d_off = torch.full((n + 1,), -7, dtype=torch.int64, device="cuda")
        st = f(C.c_void_p(d_counts.data_ptr()), n, C.c_void_p(d_off.data_ptr()),
               C.c_void_p(stream))
        assert st == ISS_OK, native.lib().iss_gpu_status_string(st)
        torch.cuda.synchronize()
        outs.append(d_off.cpu().numpy())
    return outs


@pytest.mark.gpu
def test_noalloc_scan_matches_generate_offsets():
    surf = S.viscous_3d(4000, seed=11)
    s = iSS(".", inputfile="")
    params = dict(S.DEFAULT_PARAMETERS, hydro_mode=2, afterburner_type=0,
                  include_deltaf_shear=1, include_deltaf_bulk=1, bulk_deltaf_kind=11,
                  turn_on_bulk=1, number_of_repeated_sampling=300)
    s.set_params(**params)
    s.set_surface(surf.fo_surf())
    s.set_random_seed(4242)
    s.generate_samples()
    counts = s.counts()                       # existing entry point: iss_gpu_copy_counts
    hadrons, ev_off = s.all_hadrons()         # existing entry point: iss_gpu_copy_all
    nev, nsp = counts.shape
    flat = counts.reshape(-1)
    expect = np.concatenate([[0], np.cumsum(flat, dtype=np.int64)])
    for off in _scan_twice(flat):
        np.testing.assert_array_equal(off[::nsp], ev_off)
        np.testing.assert_array_equal(off, expect)
        assert off[-1] == len(hadrons)
    s.close()


@pytest.mark.gpu
def test_noalloc_scan_takes_no_device_memory_after_the_first_call():
    """After the first call on the device (which loads the fixed array's
    module), further calls leave the device's free memory unchanged: the
    entry point itself allocates nothing."""
    import torch
    f = _fn()
    counts = np.random.default_rng(3).integers(0, 50, size=1_000_000).astype(np.int32)
    d_counts = torch.from_numpy(counts).cuda()
    d_off = torch.empty(counts.size + 1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    args = (C.c_void_p(d_counts.data_ptr()), counts.size, C.c_void_p(d_off.data_ptr()),
            C.c_void_p(stream))
    assert f(*args) == ISS_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        assert f(*args) == ISS_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    np.testing.assert_array_equal(d_off.cpu().numpy(),
                                  np.concatenate([[0], np.cumsum(counts, dtype=np.int64)]))


@pytest.mark.gpu
def test_noalloc_scan_many_tiles():
    rng = np.random.default_rng(5)
    counts = rng.integers(0, 200, size=3_000_001).astype(np.int32)   # 733 tiles
    expect = np.concatenate([[0], np.cumsum(counts, dtype=np.int64)])
    for off in _scan_twice(counts):
        np.testing.assert_array_equal(off, expect)
    (empty,) = _scan_twice(np.zeros(0, dtype=np.int32))[:1]
    assert empty.tolist() == [0]
