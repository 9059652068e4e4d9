#!/usr/bin/env python3
"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run where the reference tree is at $ISS_REFERENCE (default: a directory
named `reference` beside this repository):

    python tests/golden/make_golden.py

It compiles the unmodified reference sources with the recipe in oracle/Makefile
(`make -C oracle ref`, outputs in oracle/_ref/), then for each case:
  * writes a small synthetic MUSIC surface (iss_gb300.surfaces) into a run
    directory whose iSS_tables/ links to the reference's tables;
  * runs oracle/_ref/ref_driver `yields`, which calls the reference's own
    iSS::read_in_FO_surface and FSSW::calculate_dN_dxtdy_for_one_particle_species,
    and stores species, local-rest-frame cells and per-cell FP64 yields;
  * for the sampling cases, runs ref_driver `sample` (iSS::shell) and stores
    histograms of the reference's sampled hadrons;
  * for the writers, runs ref_driver `write` on a fixed hadron list, which
    calls the reference's own OSCAR, gzip and binary writers, and stores
    their files (the gzip file decompressed).
The GPU tests never read the reference: they only read the .npz files written
here.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
from iss_gb300 import surfaces as S  # noqa: E402

REF = os.environ.get("ISS_REFERENCE", os.path.normpath(os.path.join(REPO, os.pardir, "reference")))
REF_TABLES = os.path.join(REF, "iSS_tables")
DRIVER = os.path.join(REPO, "oracle", "_ref", "ref_driver")

# pT / y / phi binning shared with tests/test_gpu_statistics.py
PT_EDGES = np.linspace(0.0, 3.0, 61)
Y_EDGES = np.linspace(-6.0, 6.0, 61)
PHI_EDGES = np.linspace(-np.pi, np.pi, 37)
HIST_PIDS = [211, -211, 111, 321, 2212, -2212, 3122]


def build_reference():
    subprocess.check_call(["make", "-C", os.path.join(REPO, "oracle"), "ref", "-j8"],
                          stdout=subprocess.DEVNULL)


def make_run_dir(root: str) -> str:
    """Run directory: iSS_tables links to the reference tables, plus the
    header-only EOS files read_in_HRG_EOS opens unconditionally
    (src/readindata.cpp:913-936)."""
    tables = os.path.join(root, "iSS_tables")
    os.makedirs(tables)
    for name in os.listdir(REF_TABLES):
        if name != "EOS_tables":
            os.symlink(os.path.join(REF_TABLES, name), os.path.join(tables, name))
    eos = os.path.join(tables, "EOS_tables")
    os.makedirs(eos)
    for name in os.listdir(os.path.join(REF_TABLES, "EOS_tables")):
        os.symlink(os.path.join(REF_TABLES, "EOS_tables", name), os.path.join(eos, name))
    for dummy in ("SMASH.dat", "urqmd_v3.3+.dat"):
        with open(os.path.join(eos, dummy), "w") as f:
            f.write("# e P s T\n")
    with open(os.path.join(root, "s95pv1.dat"), "w") as f:
        f.write("# e P s T\n")
    os.makedirs(os.path.join(root, "work"))
    return root


def run_driver(run: str, mode: str, params: dict, out: str, timeout: int = 3600):
    pfile = os.path.join(run, "params.dat")
    S.write_parameters(pfile, **params)
    cmd = [DRIVER, mode, pfile, "work", "surface.dat", "iSS_tables", out]
    res = subprocess.run(cmd, cwd=run, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                         timeout=timeout)
    if res.returncode != 0:
        raise RuntimeError(f"ref_driver {mode} failed:\n{res.stdout.decode()[-3000:]}")
    return res.stdout.decode()


def read_yields(path):
    with open(path, "rb") as f:
        magic, n_sp = np.frombuffer(f.read(8), dtype="<i4")
        n_cells = int(np.frombuffer(f.read(8), dtype="<i8")[0])
        dt = np.dtype([("pid", "<i4"), ("idx", "<i4"), ("mass", "<f8"), ("gspin", "<i4"),
                       ("baryon", "<i4"), ("strange", "<i4"), ("charge", "<i4"), ("sign", "<i4")])
        sp = np.frombuffer(f.read(dt.itemsize * n_sp), dtype=dt)
        cells = np.frombuffer(f.read(4 * 28 * n_cells), dtype="<f4").reshape(n_cells, 28)
        y = np.frombuffer(f.read(8 * n_sp * n_cells), dtype="<f8").reshape(n_sp, n_cells)
    assert magic == 0x59494C44
    return sp, cells.copy(), y.copy()


def read_hadrons(path):
    with open(path, "rb") as f:
        magic, nev = np.frombuffer(f.read(8), dtype="<i4")
        assert magic == 0x48414452
        dt = np.dtype([("pid", "<i4"), ("mass", "<f4"), ("E", "<f4"), ("px", "<f4"),
                       ("py", "<f4"), ("pz", "<f4"), ("t", "<f4"), ("x", "<f4"),
                       ("y", "<f4"), ("z", "<f4")])
        events = []
        for _ in range(nev):
            n = int(np.frombuffer(f.read(4), dtype="<i4")[0])
            events.append(np.frombuffer(f.read(dt.itemsize * n), dtype=dt))
    return events


def histograms(events, pids):
    allh = np.concatenate(events) if events else np.zeros(0)
    out = {"n_events": len(events)}
    for pid in pids:
        h = allh[allh["pid"] == pid]
        px, py, pz, E = (h[k].astype(np.float64) for k in ("px", "py", "pz", "E"))
        pT = np.hypot(px, py)
        y = 0.5 * np.log((E + pz) / (E - pz))
        phi = np.arctan2(py, px)
        out[f"pt_{pid}"] = np.histogram(pT, PT_EDGES)[0]
        out[f"y_{pid}"] = np.histogram(y, Y_EDGES)[0]
        out[f"phi_{pid}"] = np.histogram(phi, PHI_EDGES)[0]
        out[f"v2num_{pid}"] = np.histogram(pT, PT_EDGES, weights=np.cos(2 * phi))[0]
        out[f"n_{pid}"] = np.array([np.count_nonzero(ev["pid"] == pid) for ev in events])
    return out


def yield_case(name, surface, params, work_root, cell_stride=1):
    rec = surface.records[::cell_stride].copy()
    run = make_run_dir(os.path.join(work_root, name))
    S.write_music_binary(os.path.join(run, "work", "surface.dat"), rec)
    S.write_music_input(os.path.join(run, "work"), surface)
    out = os.path.join(run, "yields.bin")
    run_driver(run, "yields", params, out)
    sp, cells, y = read_yields(out)
    np.savez_compressed(os.path.join(HERE, f"yields_{name}.npz"), records=rec,
                        hydro_mode=surface.hydro_mode, eos=surface.eos,
                        music=np.array([surface.bulk, surface.rhob, surface.diff]),
                        params=json.dumps(params), species=sp, lrf=cells, yields=y)
    print(f"{name}: {len(sp)} species x {cells.shape[0]} cells, "
          f"sum dN = {y.sum():.6e}")


def sample_case(name, surface, params, work_root):
    run = make_run_dir(os.path.join(work_root, "s_" + name))
    S.write_music_binary(os.path.join(run, "work", "surface.dat"), surface.records)
    S.write_music_input(os.path.join(run, "work"), surface)
    out = os.path.join(run, "hadrons.bin")
    run_driver(run, "sample", params, out)
    events = read_hadrons(out)
    h = histograms(events, HIST_PIDS)
    np.savez_compressed(os.path.join(HERE, f"samples_{name}.npz"), records=surface.records,
                        hydro_mode=surface.hydro_mode, eos=surface.eos,
                        music=np.array([surface.bulk, surface.rhob, surface.diff]),
                        params=json.dumps(params), pt_edges=PT_EDGES, y_edges=Y_EDGES,
                        phi_edges=PHI_EDGES, **h)
    tot = sum(len(e) for e in events)
    print(f"{name}: {len(events)} events, {tot} hadrons")


def lcc_case(visc_params, work_root):
    """local_charge_conservation = 1: positive hadrons with partners."""
    sample_case("viscous_lcc", S.viscous_3d(256, seed=2),
                dict(visc_params, local_charge_conservation=1, number_of_repeated_sampling=30000,
                     randomSeed=14), work_root)


def decays_case(visc_params, work_root):
    """perform_decays = 1: final-state hadrons after the resonance decays."""
    sample_case("viscous_decays", S.viscous_3d(256, seed=2),
                dict(visc_params, perform_decays=1, number_of_repeated_sampling=20000,
                     randomSeed=15), work_root)


def writer_hadrons(seed=31):
    """A fixed hadron list for the writer fixtures: seven events of 0 to 40
    hadrons (empty events included) whose fields cover what the formats must
    carry -- ordinary momenta and positions, signed zeros, denormals, values
    near the float limits, powers of ten and their neighbours -- and PDG
    ids of both signs."""
    rng = np.random.default_rng(seed)
    counts = [3, 0, 25, 1, 0, 40, 7]
    dt = np.dtype([("pid", "<i4"), ("mass", "<f4"), ("E", "<f4"), ("px", "<f4"),
                   ("py", "<f4"), ("pz", "<f4"), ("t", "<f4"), ("x", "<f4"),
                   ("y", "<f4"), ("z", "<f4")])
    special = np.array([0.0, -0.0, 1e-40, -3e-42, 3.4028235e38, -1.1754944e-38, 1e-7, 9.999999e-8,
                        1e16, 9.999999e16, 1e17, 1.0000001e17, 0.1, 1.0 / 3.0, 2.0 ** -149,
                        123456.79], dtype=np.float32)
    pids = np.array([211, -211, 111, 321, -321, 2212, -2212, 3122, -3334, 22], dtype=np.int32)
    events = []
    k = 0
    for n in counts:
        ev = np.zeros(n, dtype=dt)
        ev["pid"] = pids[rng.integers(0, len(pids), n)]
        for f in dt.names[1:]:
            v = (rng.standard_normal(n) * 10.0 ** rng.integers(-3, 4, n)).astype(np.float32)
            pick = rng.random(n) < 0.25
            v[pick] = special[(k + np.arange(pick.sum())) % len(special)]
            k += int(pick.sum())
            ev[f] = v
        events.append(ev)
    return events


def writers_case(work_root):
    """The reference's OSCAR, gzip and binary writers on a fixed hadron list."""
    import gzip
    events = writer_hadrons()
    run = make_run_dir(os.path.join(work_root, "writers"))
    surf = S.viscous_3d(16, seed=2)
    S.write_music_binary(os.path.join(run, "work", "surface.dat"), surf.records)
    S.write_music_input(os.path.join(run, "work"), surf)
    inp = os.path.join(run, "hadrons_in.bin")
    with open(inp, "wb") as f:
        f.write(np.array([0x48414452, len(events)], dtype="<i4").tobytes())
        for ev in events:
            f.write(np.array([len(ev)], dtype="<i4").tobytes())
            f.write(ev.tobytes())
    run_driver(run, "write", dict(hydro_mode=2, afterburner_type=0), inp)
    oscar = open(os.path.join(run, "OSCAR.DAT"), "rb").read()
    gz_text = gzip.open(os.path.join(run, "particle_samples.gz"), "rb").read()
    binary = open(os.path.join(run, "particle_samples.bin"), "rb").read()
    off = np.concatenate([[0], np.cumsum([len(e) for e in events])]).astype(np.int64)
    np.savez_compressed(os.path.join(HERE, "writers_reference.npz"),
                        hadrons=np.concatenate(events), event_offsets=off,
                        oscar=np.frombuffer(oscar, dtype=np.uint8),
                        gzip_text=np.frombuffer(gz_text, dtype=np.uint8),
                        binary=np.frombuffer(binary, dtype=np.uint8))
    print(f"writers: {off[-1]} hadrons in {len(events)} events; OSCAR {len(oscar)} B, "
          f"gzip text {len(gz_text)} B, binary {len(binary)} B")


# keys the reference's EmissionFunctionArray path (MC_sampling = 2) reads,
# with the values of its own iSS_parameters.dat
EFA_KEYS = dict(MC_sampling=2, restrict_deltaf=1, deltaf_max_ratio=1.0, sample_pT_up_to=-1,
                sample_y_minus_eta_s_range=3, use_historic_flow_output_format=0, use_pos_dN_only=0,
                minimum_emission_function_val=1e-30, calculate_vn_to_order=9, output_dN_dxtdy_4all=0,
                calculate_dN_deta=0, calculate_dN_dphi=0, calculate_dN_dtau=0, calculate_dN_dx=0,
                calculate_dN_dxt=0, bin_dtau=0.2, bin_dx=0.5, bin_tau0=0.6, bin_tau_max=17.0,
                bin_x_max=10.0, bin_x_min=-10.0)


def efa_cases(work_root, events_visc=20000, events_ideal=400):
    """MC_sampling = 2 (EmissionFunctionArray::sample_using_dN_dxtdy_4all_particles_
    conventional): lab-frame rejection with the estimated maximum."""
    sample_case("efa_viscous_rta", S.viscous_3d(256, seed=2),
                dict(EFA_KEYS, hydro_mode=2, afterburner_type=0, include_deltaf_shear=1,
                     include_deltaf_bulk=1, bulk_deltaf_kind=1, turn_on_bulk=1,
                     number_of_repeated_sampling=events_visc, randomSeed=16), work_root)
    sample_case("efa_ideal_boost_invariant", S.ideal_boost_invariant(),
                dict(EFA_KEYS, hydro_mode=1, afterburner_type=0, include_deltaf_shear=1,
                     number_of_repeated_sampling=events_ideal, randomSeed=17), work_root)
    sample_case("efa_viscous_lcc", S.viscous_3d(256, seed=2),
                dict(EFA_KEYS, hydro_mode=2, afterburner_type=0, include_deltaf_shear=1,
                     include_deltaf_bulk=1, bulk_deltaf_kind=1, turn_on_bulk=1,
                     local_charge_conservation=1, number_of_repeated_sampling=events_visc,
                     randomSeed=18), work_root)


def main():
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default=None, help="make only this fixture (e.g. samples_viscous_lcc)")
    only = ap.parse_args().only
    build_reference()
    work_root = tempfile.mkdtemp(prefix="iss_golden_")
    visc_params = dict(hydro_mode=2, afterburner_type=0, include_deltaf_shear=1,
                       include_deltaf_bulk=1, bulk_deltaf_kind=11, turn_on_bulk=1)
    if only in ("samples_efa", "samples_efa_viscous_lcc"):
        try:
            if only == "samples_efa":
                efa_cases(work_root)
            else:
                sample_case("efa_viscous_lcc", S.viscous_3d(256, seed=2),
                            dict(EFA_KEYS, hydro_mode=2, afterburner_type=0, include_deltaf_shear=1,
                                 include_deltaf_bulk=1, bulk_deltaf_kind=1, turn_on_bulk=1,
                                 local_charge_conservation=1, number_of_repeated_sampling=20000,
                                 randomSeed=18), work_root)
        finally:
            shutil.rmtree(work_root, ignore_errors=True)
        return
    if only == "writers_reference":
        try:
            writers_case(work_root)
        finally:
            shutil.rmtree(work_root, ignore_errors=True)
        return
    if only in ("samples_viscous_lcc", "samples_viscous_decays"):
        try:
            (lcc_case if only == "samples_viscous_lcc" else decays_case)(visc_params, work_root)
        finally:
            shutil.rmtree(work_root, ignore_errors=True)
        return
    try:
        # per-cell yields
        yield_case("ideal_boost_invariant", S.ideal_boost_invariant(),
                   dict(hydro_mode=1, afterburner_type=0, include_deltaf_shear=1),
                   work_root, cell_stride=8)
        yield_case("viscous_14moment", S.viscous_3d(128, seed=2), visc_params, work_root)
        yield_case("viscous_rta", S.viscous_3d(64, seed=7),
                   dict(visc_params, bulk_deltaf_kind=1), work_root)
        yield_case("viscous_boltzmann", S.viscous_3d(48, seed=11),
                   dict(visc_params, quantum_statistics=0), work_root)
        ce = S.viscous_3d(64, seed=5)
        ce.eos = 91
        yield_case("viscous_ce_smash", ce,
                   dict(visc_params, afterburner_type=2, bulk_deltaf_kind=21), work_root)
        yield_case("diffusion_smash", S.finite_density_3d(64, seed=3),
                   dict(visc_params, afterburner_type=2, include_deltaf_diffusion=1,
                        turn_on_rhob=1, turn_on_diff=1), work_root)
        # sampled hadrons (statistics)
        static = S.viscous_3d(16, seed=21, umax=0.0)
        static.records[:, 8:12] = [1.0, 0.0, 0.0, 0.0]
        static.records[:, 4:8] = [0.03125 * 40.0, 0.0, 0.0, 0.0]
        sample_case("static_viscous", static,
                    dict(visc_params, number_of_repeated_sampling=40000, randomSeed=11),
                    work_root)
        sample_case("viscous_14moment", S.viscous_3d(256, seed=2),
                    dict(visc_params, number_of_repeated_sampling=100000, randomSeed=12),
                    work_root)
        sample_case("ideal_boost_invariant", S.ideal_boost_invariant(),
                    dict(hydro_mode=1, afterburner_type=0, include_deltaf_shear=1,
                         number_of_repeated_sampling=1000, randomSeed=13), work_root)
        lcc_case(visc_params, work_root)
        decays_case(visc_params, work_root)
        efa_cases(work_root)
        writers_case(work_root)
    finally:
        shutil.rmtree(work_root, ignore_errors=True)


if __name__ == "__main__":
    main()
