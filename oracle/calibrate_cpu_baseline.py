#!/usr/bin/env python3
"""Test infrastructure: compares the speed of the reference binary
(oracle/_ref/ref_driver, compiled from the reference's sources by
`make -C oracle ref`) with the oracle's port of the reference's sampling
algorithm (oracle part 3, the CPU baseline of bench.py) on the same cells,
species, parameters and number of events, single-threaded on this host.

    python oracle/calibrate_cpu_baseline.py [--cells-every 10] [--events 100] [--bulk-kind 1]

Needs the reference tree (ISS_REFERENCE, default: a directory named
`reference` beside this repository) for its
iSS_tables; prints one JSON line."""
from __future__ import annotations

import argparse
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "tests"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells-every", type=int, default=10)
    ap.add_argument("--events", type=int, default=100)
    ap.add_argument("--bulk-kind", type=int, default=1,
                    help="bulk delta-f kind; the default 1 avoids kind 11, whose c0 "
                         "table the reference leaves unread (uninitialised memory)")
    args = ap.parse_args()
    import oracle_lib as O
    from iss_gb300 import surfaces as S
    sys.path.insert(0, os.path.join(REPO, "tests", "golden"))
    import make_golden as G

    G.build_reference()
    surf = S.viscous_3d(200_000, seed=2)
    surf.records = surf.records[::args.cells_every].copy()
    params = dict(hydro_mode=2, afterburner_type=0, include_deltaf_shear=1,
                  include_deltaf_bulk=1, bulk_deltaf_kind=args.bulk_kind, turn_on_bulk=1,
                  number_of_repeated_sampling=args.events, randomSeed=5)
    root = tempfile.mkdtemp(prefix="iss_calib_")
    try:
        run = G.make_run_dir(os.path.join(root, "run"))
        S.write_music_binary(os.path.join(run, "work", "surface.dat"), surf.records)
        S.write_music_input(os.path.join(run, "work"), surf)
        t0 = time.perf_counter()
        log = G.run_driver(run, "sample", params, os.path.join(run, "h.bin"))
        t_ref = time.perf_counter() - t0
        events = G.read_hadrons(os.path.join(run, "h.bin"))
        n_ref = sum(len(e) for e in events)
        m = re.search(r"sample_using_dN_dxtdy_4all_particles finished in\s+([0-9.eE+-]+)", log)
        t_ref_sampling = float(m.group(1)) if m else None
    finally:
        shutil.rmtree(root, ignore_errors=True)

    fo = surf.fo_surf()
    lrf, keep = O.lrf_cells(fo)
    oc = O.OracleConfig(dict(S.DEFAULT_PARAMETERS, **params), S.TABLE_DIR, n_events=args.events)
    sp = O.chosen_species(S.TABLE_DIR, 0)
    t0 = time.perf_counter()
    _, n_port, t_port_inner = O.reference_sampler(oc, sp, lrf, keep, seed=5)
    t_port = time.perf_counter() - t0
    out = {"cells": int(fo.shape[0]), "events": args.events, "bulk_deltaf_kind": args.bulk_kind,
           "reference_binary": {"hadrons": n_ref, "wall_s": t_ref,
                                "sampling_phase_cpu_s": t_ref_sampling,
                                "hadrons_per_s_wall": n_ref / t_ref},
           "oracle_port": {"hadrons": int(n_port), "wall_s": t_port,
                           "hadrons_per_s_wall": n_port / t_port},
           "port_speed_over_reference": (n_port / t_port) / (n_ref / t_ref)}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
