"""The output writers against files the reference's own writers produced.

tests/golden/writers_reference.npz holds a fixed hadron list (seven events,
empty ones included, with signed zeros, denormals, values near the float
limits and powers of ten) and the three files the reference wrote for it:
FSSW::combine_samples_to_OSCAR, combine_samples_to_gzip_file and
combine_samples_to_binary_file (src/FSSW.cpp:365-561), run by
oracle/ref_driver `write` on the unmodified reference (tests/golden/
make_golden.py).  iss_gpu_write_hadron_list writes the same list here with
the library's writers; OSCAR and binary files must equal the reference's
byte for byte, the gzip stream must decompress to the same bytes (the
compressed bytes depend on the zlib build and the gzip header's time field).
The OSCAR text the GPU formats is compared with the host writer's in
tests/test_gpu_parity.py, so it equals the reference's too.
"""
import gzip
import os

import numpy as np
import pytest

import oracle_lib as O
from iss_gb300 import native


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(O.REPO, "tests", "golden", "writers_reference.npz"))


def _write(tmp_path, fmt, name, g):
    fn = str(tmp_path / name)
    native.write_hadron_list(fmt, fn, g["hadrons"].view(native.HADRON_DTYPE), g["event_offsets"])
    return open(fn, "rb").read()


def test_oscar_equals_reference_bytes(tmp_path, golden):
    out = _write(tmp_path, native.OUTPUT_OSCAR, "OSCAR.DAT", golden)
    ref = golden["oscar"].tobytes()
    assert len(out) == len(ref)
    assert out == ref


def test_binary_equals_reference_bytes(tmp_path, golden):
    out = _write(tmp_path, native.OUTPUT_BINARY, "particle_samples.bin", golden)
    assert out == golden["binary"].tobytes()


def test_gzip_text_equals_reference(tmp_path, golden):
    _write(tmp_path, native.OUTPUT_GZIP, "particle_samples.gz", golden)
    text = gzip.open(str(tmp_path / "particle_samples.gz"), "rb").read()
    assert text == golden["gzip_text"].tobytes()


def test_writer_rejects_bad_offsets(tmp_path, golden):
    h = golden["hadrons"].view(native.HADRON_DTYPE)
    with pytest.raises(native.IssError):
        native.write_hadron_list(native.OUTPUT_BINARY, str(tmp_path / "x.bin"), h,
                                 np.array([0, 5, 3], dtype=np.int64))
    with pytest.raises(native.IssError):
        native.write_hadron_list(99, str(tmp_path / "x.bin"), h, golden["event_offsets"])
