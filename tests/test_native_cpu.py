"""Host-side checks of the native library that need no GPU: the library
loads and exports every entry point of include/iss_gpu.h, parameter and
surface reading follow the reference's rules, and compute calls fail loudly
without a device."""
import ctypes
import os
import re
import tempfile

import numpy as np
import pytest

import oracle_lib as O
from conftest import REPO, gpu_available
from iss_gb300 import IssError, iSS, native, surfaces as S


def declared_symbols():
    text = open(os.path.join(REPO, "include", "iss_gpu.h")).read()
    return sorted(set(re.findall(r"\b(iss_gpu_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = native.lib()
    names = declared_symbols()
    assert len(names) >= 25
    for name in names:
        assert hasattr(L, name), name
    assert set(names) == set(native.EXPORTED)


def test_status_strings():
    L = native.lib()
    assert L.iss_gpu_status_string(0) == b"ok"
    assert L.iss_gpu_status_string(5) == b"CUDA error"


def test_parameter_reader_semantics(tmp_path):
    f = tmp_path / "p.dat"
    f.write_text("Hydro_Mode = 2   # comment\n  y_LB=-4.5\nno equal sign line\n"
                 "randomSeed = 7\nrandomseed = 9\n")
    s = iSS(str(tmp_path), inputfile=str(f))
    assert s.getVal("hydro_mode") == 2
    assert s.getVal("Y_lb") == -4.5
    assert s.getVal("randomSeed") == 9          # later assignment overwrites
    with pytest.raises(IssError):
        s.getVal("not_a_key")
    assert s.getVal("not_a_key", 3.0) == 3.0
    s.readFromArguments(["y_RB = 2.5 # trailing"])
    assert s.getVal("y_rb") == 2.5


def test_missing_parameter_file_is_an_error(tmp_path):
    with pytest.raises(IssError):
        iSS(str(tmp_path), inputfile=str(tmp_path / "missing.dat"))


def _surface_dir(surf, binary=True, text_rows=None):
    d = tempfile.mkdtemp()
    if binary:
        S.write_music_binary(os.path.join(d, "surface.dat"), surf.records)
    else:
        with open(os.path.join(d, "surface.dat"), "w") as f:
            for r in text_rows:
                f.write("  ".join(repr(float(x)) for x in r) + "\n")
    S.write_music_input(d, surf, binary=binary)
    return d


def test_binary_reader_matches_reference_conversions():
    surf = S.viscous_3d(300, seed=4)
    d = _surface_dir(surf)
    s = iSS(d)
    s.set_params(**S.DEFAULT_PARAMETERS)
    s.read_in_FO_surface()
    assert s.num_cells() == 300
    pids = s.species()
    assert np.array_equal(pids, O.chosen_species(S.TABLE_DIR, 0)["pid"])


def test_text_and_binary_surfaces_agree():
    """Binary and text MUSIC surfaces give the same cells, also when columns
    are switched on by music_input."""
    surf = S.viscous_3d(40, seed=6)
    cols = list(range(28)) + [28]          # bulk column present (turn_on_bulk = 1)
    d_txt = _surface_dir(surf, binary=False, text_rows=surf.records[:, cols])
    d_bin = _surface_dir(surf)
    out = []
    for d in (d_txt, d_bin):
        s = iSS(d)
        s.set_params(**S.DEFAULT_PARAMETERS)
        s.read_in_FO_surface()
        out.append(s.num_cells())
    assert out[0] == out[1] == 40


def test_cold_cells_are_discarded():
    surf = S.viscous_3d(50, seed=8)
    surf.records[::5, 13] = 0.005 / S.HBARC     # T = 5 MeV < 10 MeV
    d = _surface_dir(surf)
    s = iSS(d)
    s.set_params(**S.DEFAULT_PARAMETERS)
    s.read_in_FO_surface()
    assert s.num_cells() == 40


def test_unsupported_options_are_reported():
    surf = S.viscous_3d(10, seed=9)
    s = iSS(".")
    s.set_params(**S.DEFAULT_PARAMETERS)
    s.set_surface(surf.fo_surf())
    s.setVal("MC_sampling", 3)
    with pytest.raises(IssError) as e:
        s.generate_samples()
    assert e.value.status in (4, 5)   # unsupported (or no CUDA device here)


def test_pce_eos_rejected():
    surf = S.viscous_3d(10, seed=9)
    surf.eos = 3
    d = _surface_dir(surf)
    s = iSS(d)
    s.set_params(**S.DEFAULT_PARAMETERS)
    with pytest.raises(IssError) as e:
        s.read_in_FO_surface()
    assert e.value.status == 4


@pytest.mark.skipif(gpu_available(), reason="checks the no-device error path")
def test_generate_without_gpu_fails_loudly():
    surf = S.viscous_3d(10, seed=9)
    s = iSS(".")
    s.set_params(**S.DEFAULT_PARAMETERS)
    s.set_surface(surf.fo_surf())
    with pytest.raises(IssError) as e:
        s.generate_samples()
    assert e.value.status == 5
