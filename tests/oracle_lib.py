"""ctypes binding of the oracle (oracle/_build/liboracle.so) and table loaders
that mirror the reference's parsing, for the tests and the CPU baseline only.

The oracle is the checker: nothing in the product (iss_gb300/) imports this
module."""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(REPO, "oracle")
LIB_PATH = os.path.join(ORACLE_DIR, "_build", "liboracle.so")
HBARC = 0.197327053
SF_LEN = 7991


def build():
    subprocess.check_call(["make", "-C", ORACLE_DIR, "-s"])


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _setup(_lib)
    return _lib


class Species(C.Structure):
    _fields_ = [("pid", C.c_int32), ("real_idx", C.c_int32), ("mass", C.c_double),
                ("gspin", C.c_int32), ("baryon", C.c_int32), ("strange", C.c_int32),
                ("charge", C.c_int32), ("sign", C.c_int32)]


class Cfg(C.Structure):
    _fields_ = [("hydro_mode", C.c_int32), ("include_shear", C.c_int32),
                ("include_bulk", C.c_int32), ("include_diff", C.c_int32),
                ("bulk_kind", C.c_int32), ("neos_kind", C.c_int32),
                ("y_lb", C.c_double), ("y_rb", C.c_double),
                ("sampling_model", C.c_int32), ("sampling_para1", C.c_double),
                ("n_events", C.c_int64), ("event_offset", C.c_int64), ("seed", C.c_uint64),
                ("compat_fermion", C.c_int32), ("max_tries", C.c_int32),
                ("max_redraws", C.c_int32), ("lcc", C.c_int32),
                ("sf_K", C.c_void_p), ("sf_E", C.c_void_p),
                ("b14_nT", C.c_int32), ("b14_nmu", C.c_int32),
                ("b14_T0", C.c_double), ("b14_mu0", C.c_double), ("b14_dT", C.c_double),
                ("b14_dmu", C.c_double), ("b14_c0", C.c_void_p), ("b14_c1", C.c_void_p),
                ("b14_c2", C.c_void_p), ("ce_tb", C.c_void_p), ("qmu_tb", C.c_void_p)]


class DParticle(C.Structure):
    _fields_ = [("pid", C.c_int32), ("mass", C.c_double), ("width", C.c_double),
                ("stable", C.c_int32), ("first_channel", C.c_int32), ("n_channels", C.c_int32)]


class DChannel(C.Structure):
    _fields_ = [("n_daughters", C.c_int32), ("daughter", C.c_int32 * 5), ("cum53", C.c_uint64)]


class Stats(C.Structure):
    _fields_ = [("n_tries", C.c_int64), ("n_redraws", C.c_int64), ("n_failures", C.c_int64),
                ("n_bound_violations", C.c_int64)]


HADRON_DTYPE = np.dtype([("pid", "<i4"), ("mass", "<f4"), ("E", "<f4"), ("px", "<f4"),
                         ("py", "<f4"), ("pz", "<f4"), ("t", "<f4"), ("x", "<f4"),
                         ("y", "<f4"), ("z", "<f4")])
SPECIES_DTYPE = np.dtype([("pid", "<i4"), ("idx", "<i4"), ("mass", "<f8"), ("gspin", "<i4"),
                          ("baryon", "<i4"), ("strange", "<i4"), ("charge", "<i4"),
                          ("sign", "<i4")])


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _setup(L):
    v = C.c_void_p
    L.orc_sf_tables.argtypes = [C.c_int, C.c_int, v, v]
    L.orc_lrf_cells.argtypes = [v, C.c_int64, v, v]
    L.orc_cell_coeffs.argtypes = [C.POINTER(Cfg), v, C.c_int64, v]
    L.orc_yields.argtypes = [C.POINTER(Cfg), v, C.c_int32, v, v, C.c_int64, v]
    L.orc_yields.restype = C.c_int
    L.orc_cdf.argtypes = [v, C.c_int32, C.c_int64, v, v, v]
    L.orc_counts.argtypes = [C.POINTER(Cfg), v, C.c_int32, v, v]
    L.orc_counts.restype = C.c_int
    L.orc_sample_replay.argtypes = [C.POINTER(Cfg), v, C.c_int32, v, C.c_int64, v, v, v, v,
                                    v, C.c_int64, C.POINTER(Stats)]
    L.orc_sample_replay.restype = C.c_int64
    L.orc_decay_replay.argtypes = [v, C.c_int32, v, C.c_uint64, C.c_int64, C.c_int32, v, v,
                                   C.c_int64, v, v, C.POINTER(C.c_int64)]
    L.orc_decay_replay.restype = C.c_int64
    if hasattr(L, "orc_reference_sampler"):
        L.orc_reference_sampler.argtypes = [C.POINTER(Cfg), v, C.c_int32, v, v, C.c_int64,
                                            C.c_int32, C.c_uint64, v, C.c_int64,
                                            C.POINTER(C.c_double)]
        L.orc_reference_sampler.restype = C.c_int64


# ---------------------------------------------------------------------------
# table loaders with the reference's parsing rules

def chosen_species(table_dir, afterburner, quantum_statistics=1):
    """Mass-sorted chosen species exactly as FSSW builds them:
    read_resonances_list (src/readindata.cpp:971-1116), the chosen table
    (src/iSS.cpp:133-142, src/FSSW.cpp:115-149) and the stable bubble sort by
    mass (src/FSSW.cpp:151-162)."""
    name = {2: "pdg-SMASH.dat", 1: "pdg-urqmd_v3.3+.dat"}.get(afterburner, "pdg-s95pv1.dat")
    cname = {2: "chosen_particles_SMASH.dat", 1: "chosen_particles_urqmd_v3.3+.dat"}.get(
        afterburner, "chosen_particles_s95p-v1.dat")
    particles = []
    lines = open(os.path.join(table_dir, name)).read().split("\n")
    i = 0
    while i < len(lines):
        tok = lines[i].split()
        if len(tok) < 12:
            i += 1
            continue
        pid, mass, g, B, S, Q, nd = (int(tok[0]), float(tok[2]), int(tok[4]), int(tok[5]),
                                     int(tok[6]), int(tok[10]), int(tok[11]))
        particles.append((pid, mass, g, B, S, Q))
        if B > 0:
            particles.append((-pid, mass, g, -B, -S, -Q))
        i += 1 + nd
    chosen = [int(float(t)) for t in open(os.path.join(table_dir, cname)).read().split()]
    table = []
    for mon in chosen:
        for n, p in enumerate(particles):
            if p[0] == mon:
                table.append(n)
                break
    nc = len(table)
    for m in range(nc):
        for n in range(nc - m - 1):
            if particles[table[n]][1] > particles[table[n + 1]][1]:
                table[n], table[n + 1] = table[n + 1], table[n]
    out = np.zeros(nc, dtype=SPECIES_DTYPE)
    for k, n in enumerate(table):
        pid, mass, g, B, S, Q = particles[n]
        sign = (-1 if B == 0 else 1) if quantum_statistics else 0
        out[k] = (pid, n, mass, g, B, S, Q, sign)
    return out


def load_b14(table_dir, afterburner, fix_c0=False):
    """OSU 14-moment tables as load_bulk_deltaf_14mom_table reads them
    (src/FSSW.cpp:1215-1300).  The reference reads c0.dat's two size lines
    but not its column-title line, so every c0 read fails and c0 stays zero;
    fix_c0=True reads the c0 column instead."""
    folder = "smash_box" if afterburner == 2 else "urqmd"
    d = os.path.join(table_dir, "deltaf_tables", folder)

    def read(fn):
        with open(os.path.join(d, fn)) as f:
            nT = int(f.readline())
            nmu = int(f.readline())
            f.readline()
            a = np.loadtxt(f)
        return nT, nmu, a

    nT, nmu, a1 = read("c1.dat")
    _, _, a2 = read("c2.dat")
    _, _, a0 = read("c0.dat")
    shape = (nmu, nT)
    c1 = a1[:, 2].reshape(shape).T.copy()
    c2 = a2[:, 2].reshape(shape).T.copy()
    c0 = a0[:, 2].reshape(shape).T.copy() if fix_c0 else np.zeros((nT, nmu))
    T0, mu0 = a2[0, 0], a2[0, 1]
    dT = a2[1, 0] - T0
    dmu = a2[nT, 1] - mu0
    return dict(nT=nT, nmu=nmu, T0=T0, mu0=mu0, dT=dT, dmu=dmu, c0=c0, c1=c1, c2=c2)


def load_ce(table_dir, afterburner):
    folder = "smash" if afterburner == 2 else "urqmd"
    return np.loadtxt(os.path.join(table_dir, "deltaf_tables", folder,
                                   "NEoSBQS_CE_deltafCoeff.dat"), skiprows=1)


def load_qmu(table_dir):
    a = np.loadtxt(os.path.join(table_dir, "deltaf_tables", "Coefficients_RTA_diffusion.dat"))
    return a[:, 2].reshape(100, 150).T.copy()


class OracleConfig:
    """Builds the oracle's configuration (and keeps its arrays alive)."""

    def __init__(self, params: dict, table_dir: str, afterburner=None, n_events=None,
                 seed=1, compat_fermion=0, max_tries=10000, max_redraws=64, fix_c0=False,
                 event_offset=0):
        p = {k.lower(): v for k, v in params.items()}
        self.p = p
        ab = int(p.get("afterburner_type", 0)) if afterburner is None else afterburner
        self.afterburner = ab
        c = Cfg()
        c.hydro_mode = int(p.get("hydro_mode", 2))
        c.include_shear = int(p.get("include_deltaf_shear", 0))
        c.include_bulk = int(p.get("include_deltaf_bulk", 0))
        c.include_diff = int(p.get("include_deltaf_diffusion", 0))
        c.bulk_kind = int(p.get("bulk_deltaf_kind", 1))
        c.neos_kind = {21: 1, 20: 0}.get(c.bulk_kind, -1)
        c.y_lb = float(p.get("y_lb", -5.0))
        c.y_rb = float(p.get("y_rb", 5.0))
        c.sampling_model = int(p.get("dn_dy_sampling_model", 30))
        c.sampling_para1 = float(p.get("dn_dy_sampling_para1", 0.16))
        c.n_events = int(p.get("number_of_repeated_sampling", 1) if n_events is None else n_events)
        c.event_offset = int(event_offset)
        c.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        c.compat_fermion = int(compat_fermion)
        c.max_tries = max_tries
        c.max_redraws = max_redraws
        c.lcc = int(int(p.get("local_charge_conservation", 0)) == 1)
        L = lib()
        self.sf_K = np.zeros(SF_LEN * 3)
        self.sf_E = np.zeros(SF_LEN * 9)
        L.orc_sf_tables(c.include_bulk, c.include_diff, _p(self.sf_K), _p(self.sf_E))
        c.sf_K, c.sf_E = _p(self.sf_K), _p(self.sf_E)
        if c.include_bulk and c.bulk_kind == 11:
            b = load_b14(table_dir, ab, fix_c0=fix_c0)
            self.b14 = b
            c.b14_nT, c.b14_nmu = b["nT"], b["nmu"]
            c.b14_T0, c.b14_mu0, c.b14_dT, c.b14_dmu = b["T0"], b["mu0"], b["dT"], b["dmu"]
            c.b14_c0, c.b14_c1, c.b14_c2 = _p(b["c0"]), _p(b["c1"]), _p(b["c2"])
        if c.neos_kind == 1:
            self.ce = np.ascontiguousarray(load_ce(table_dir, ab))
            c.ce_tb = _p(self.ce)
        if c.include_diff:
            self.qmu = load_qmu(table_dir)
            c.qmu_tb = _p(self.qmu)
        self.cfg = c


def species_array(sp):
    arr = (Species * len(sp))()
    for k, s in enumerate(sp):
        arr[k] = Species(int(s["pid"]), int(s["idx"]), float(s["mass"]), int(s["gspin"]),
                         int(s["baryon"]), int(s["strange"]), int(s["charge"]), int(s["sign"]))
    return arr


def lrf_cells(fo34):
    fo34 = np.ascontiguousarray(fo34, dtype=np.float32)
    n = fo34.shape[0]
    out = np.zeros((n, 28), dtype=np.float32)
    keep = np.zeros(n, dtype=np.int32)
    lib().orc_lrf_cells(_p(fo34), n, _p(out), _p(keep))
    return out, keep


def cell_coeffs(oc: OracleConfig, lrf):
    lrf = np.ascontiguousarray(lrf, dtype=np.float32)
    out = np.zeros((lrf.shape[0], 4))
    lib().orc_cell_coeffs(C.byref(oc.cfg), _p(lrf), lrf.shape[0], _p(out))
    return out


def yields(oc: OracleConfig, sp, lrf, keep=None):
    lrf = np.ascontiguousarray(lrf, dtype=np.float32)
    n = lrf.shape[0]
    arr = species_array(sp)
    out = np.zeros((len(sp), n))
    kp = None if keep is None else np.ascontiguousarray(keep, dtype=np.int32)
    st = lib().orc_yields(C.byref(oc.cfg), C.cast(arr, C.c_void_p), len(sp), _p(lrf),
                          None if kp is None else _p(kp), n, _p(out))
    if st != 0:
        raise RuntimeError(f"orc_yields status {st}")
    return out


def cdf(yields_f32):
    """Fixed-point cell CDF of the GPU sampler: (rows, totals), rows uint64
    (n_species, n_cells + 1) with rows[:, -1] the integer totals Q."""
    y = np.ascontiguousarray(yields_f32, dtype=np.float32)
    n_sp, n = y.shape
    c = np.zeros((n_sp, n + 1), dtype=np.uint64)
    q = np.zeros(n_sp, dtype=np.uint64)
    tot = np.zeros(n_sp)
    lib().orc_cdf(_p(y), n_sp, n, _p(c), _p(q), _p(tot))
    return c, tot


def counts(oc: OracleConfig, sp, totals):
    arr = species_array(sp)
    tot = np.ascontiguousarray(totals, dtype=np.float64)
    out = np.zeros((oc.cfg.n_events, len(sp)), dtype=np.int32)
    st = lib().orc_counts(C.byref(oc.cfg), C.cast(arr, C.c_void_p), len(sp), _p(tot), _p(out))
    if st != 0:
        raise RuntimeError(f"orc_counts status {st}")
    return out


def sample_replay(oc: OracleConfig, sp, lrf, coef4, cdf_rows, cnt):
    arr = species_array(sp)
    lrf = np.ascontiguousarray(lrf, dtype=np.float32)
    coef = np.ascontiguousarray(coef4, dtype=np.float32)
    cdf_rows = np.ascontiguousarray(cdf_rows, dtype=np.uint64)
    qtot = np.ascontiguousarray(cdf_rows[:, -1])
    cnt = np.ascontiguousarray(cnt, dtype=np.int32)
    cap = int(cnt.sum())
    out = np.zeros(max(cap, 1), dtype=HADRON_DTYPE)
    st = Stats()
    n = lib().orc_sample_replay(C.byref(oc.cfg), C.cast(arr, C.c_void_p), len(sp), _p(lrf),
                                lrf.shape[0], _p(coef), _p(cdf_rows), _p(qtot), _p(cnt),
                                _p(out), cap, C.byref(st))
    if n < 0:
        raise RuntimeError(f"orc_sample_replay status {n}")
    return out[:n], st


def decay_table(table_dir, afterburner):
    """The decay table as particle_decay::read_resonances_list reads the pdg
    file (src/particle_decay.cpp:33-160), restated: whitespace tokens
    (pid, name, mass, width, g, B, S, charm, bottom, g_iso, Q, n_channels,
    then per channel: pid, n_daughters, branching ratio, 5 daughter pids);
    stable when the first channel has one daughter; every baryon (B = 1) is
    followed by its anti-baryon, whose daughters are negated unless the
    first entry read so far with that pid is a neutral non-strange meson.
    Daughters become indices of the first entry with their pid (-1 unknown);
    cum53 = ceil(2^53 x the FP64 partial sum of branching ratios)."""
    import math
    name = {2: "pdg-SMASH.dat", 1: "pdg-urqmd_v3.3+.dat"}.get(afterburner, "pdg-s95pv1.dat")
    tok = open(os.path.join(table_dir, name)).read().split()
    parts = []   # [pid, mass, width, B, S, Q, stable, channels]
    k = 0
    while k + 12 <= len(tok):
        pid = int(tok[k])
        mass, width = float(tok[k + 2]), float(tok[k + 3])
        B, S, Q, nd = int(tok[k + 5]), int(tok[k + 6]), int(tok[k + 10]), int(tok[k + 11])
        k += 12
        ch = []
        for _ in range(nd):
            npart, br = int(tok[k + 1]), float(tok[k + 2])
            ch.append((npart, br, [int(t) for t in tok[k + 3:k + 8]]))
            k += 8
        stable = 1 if ch and ch[0][0] == 1 else 0
        parts.append([pid, mass, width, B, S, Q, stable, ch])
        if B == 1:
            anti = []
            for npart, br, ds in ch:
                nds = []
                for d in ds:
                    if d == 0:
                        nds.append(0)
                        continue
                    hit = next((p for p in parts if p[0] == d), None)
                    neutral = hit is not None and hit[3] == 0 and hit[5] == 0 and hit[4] == 0
                    nds.append(d if neutral else -d)
                anti.append((npart, br, nds))
            parts.append([-pid, mass, width, -B, -S, -Q, stable, anti])
    first = {}
    for i, p in enumerate(parts):
        first.setdefault(p[0], i)
    dp = (DParticle * len(parts))()
    chans = []
    for i, p in enumerate(parts):
        dp[i].pid, dp[i].mass, dp[i].width, dp[i].stable = p[0], p[1], p[2], p[6]
        dp[i].first_channel, dp[i].n_channels = len(chans), len(p[7])
        cum = 0.0
        for npart, br, ds in p[7]:
            cum += br
            x = math.ceil(math.ldexp(cum, 53))
            c = DChannel()
            c.n_daughters = npart
            for j in range(5):
                c.daughter[j] = first.get(ds[j], -1) if (j < npart and ds[j] != 0) else -1
            c.cum53 = 0 if x <= 0 else min(x, 2 ** 64 - 1)
            chans.append(c)
    dc = (DChannel * max(len(chans), 1))(*chans)
    return dp, dc


def decay_replay(table, seed, ev_off, hadrons, event_offset=0):
    """Final-state lists of the events whose sampled hadrons are
    hadrons[ev_off[e]:ev_off[e + 1]] (oracle_decay.c); returns (records,
    event offsets, 3-body failures)."""
    dp, dc = table
    ev_off = np.ascontiguousarray(ev_off, dtype=np.int64)
    had = np.ascontiguousarray(hadrons, dtype=HADRON_DTYPE)
    n_ev = len(ev_off) - 1
    cap = 4 * max(len(had), 1) + 64
    while True:
        out = np.zeros(cap, dtype=HADRON_DTYPE)
        off = np.zeros(n_ev + 1, dtype=np.int64)
        fails = C.c_int64(0)
        n = lib().orc_decay_replay(C.cast(dp, C.c_void_p), len(dp), C.cast(dc, C.c_void_p),
                                   int(seed) & 0xFFFFFFFFFFFFFFFF, int(event_offset), n_ev,
                                   _p(ev_off), _p(had), cap, _p(out), _p(off), C.byref(fails))
        if n == -1:
            cap *= 2
            continue
        if n < 0:
            raise RuntimeError(f"orc_decay_replay status {n}")
        return out[:n], off, int(fails.value)


def load_golden(name):
    path = os.path.join(REPO, "tests", "golden", name)
    z = np.load(path, allow_pickle=False)
    d = {k: z[k] for k in z.files}
    d["params"] = json.loads(str(d["params"]))
    return d


def reference_sampler(oc: OracleConfig, sp, lrf, keep, seed=1, capacity=None):
    """The reference's own sampling algorithm (oracle part 3); returns
    (hadrons, seconds)."""
    arr = species_array(sp)
    lrf = np.ascontiguousarray(lrf, dtype=np.float32)
    kp = np.ascontiguousarray(keep, dtype=np.int32)
    cap = int(capacity) if capacity is not None else 0
    out = np.zeros(max(cap, 1), dtype=HADRON_DTYPE)
    sec = C.c_double()
    n = lib().orc_reference_sampler(C.byref(oc.cfg), C.cast(arr, C.c_void_p), len(sp), _p(lrf),
                                    _p(kp), lrf.shape[0], 1, seed, _p(out) if cap else None, cap,
                                    C.byref(sec))
    if n < 0:
        raise RuntimeError(f"orc_reference_sampler status {n}")
    return out[:min(n, cap)], n, sec.value


def events_needed(params: dict, sp, yields_fp64):
    """FSSW::compute_number_of_sampling_needed (src/FSSW.cpp:851-869): the
    number of events from the thermal pi+ yield (the species whose table
    index is 1, summed over cells in FP64), number_of_particles_needed and
    maximum_sampling_events; ten times more for 3+1D surfaces."""
    p = {k.lower(): v for k, v in params.items()}
    k = [i for i, s in enumerate(sp) if int(s["idx"]) == 1][0]
    dn_pion = float(np.sum(yields_fp64[k]))
    needed = int(float(p["number_of_particles_needed"]))     # the reference's long
    nev = int(needed / (6.0 * dn_pion))
    if int(p.get("hydro_mode", 2)) == 2:
        nev *= 10
    return max(1, min(int(float(p["maximum_sampling_events"])), nev))
