"""Synthetic MUSIC freeze-out surfaces and run directories.

The benchmark workloads have no public data set: they are seeded synthetic
surfaces with the shapes, sizes and value ranges of the workloads the sampler
is quoted on.  This module builds them as MUSIC records (34 floats per cell in
the units of MUSIC's binary surface file, the layout read at
src/readindata.cpp:645-689) and converts them to the reference's FO_surf
records (src/data_struct.h:53-63) with the same float arithmetic as the
reference's reader, so that the in-memory entry point and the file reader see
identical cells.

Workloads (sizes in the names):
  * ideal_boost_invariant  -- 1,245 cells, boost-invariant (hydro_mode 1),
    tau_f = 10 fm, 0.5 fm grid, r < 10 fm, T = 0.150 GeV, u^r = 0.6 r/10 fm.
  * viscous_3d             -- 200,000 cells on 64 eta slices in [-4, 4],
    tau in [8, 14] fm, T in [0.145, 0.155] GeV, Bjorken + radial flow up to
    0.75, 20 % spacelike cells with |dsigma_perp|/dsigma_tau in [0, 1.5],
    random transverse-traceless shear with |pi|/(e+P) in [0, 0.3], bulk
    Pi/(e+P) in [-0.1, 0].
  * finite_density_3d      -- 1,000,000 cells like viscous_3d with T in
    [0.130, 0.155] GeV, mu_B in [0, 0.4] GeV and baryon diffusion orthogonal to
    u with |q|/n_B <= 0.2.
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np

HBARC = 0.197327053
DATA_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
TABLE_DIR = os.path.join(DATA_DIR, "iSS_tables")

__all__ = [
    "HBARC", "TABLE_DIR", "Surface", "ideal_boost_invariant", "viscous_3d",
    "finite_density_3d", "music_to_fo_surf", "write_music_binary",
    "write_music_input", "write_parameters", "load_species", "hrg_thermo",
]


@dataclass
class Surface:
    """MUSIC records (float32 [n, 34], file units) plus how to read them."""
    records: np.ndarray
    hydro_mode: int
    eos: int = 2
    bulk: int = 0
    rhob: int = 0
    diff: int = 0

    @property
    def n_cells(self) -> int:
        return int(self.records.shape[0])

    def fo_surf(self) -> np.ndarray:
        return music_to_fo_surf(self.records, self.hydro_mode)


# --------------------------------------------------------------------------
# species lists and a hadron-resonance-gas equation of state

def load_species(table_dir: str = TABLE_DIR, afterburner: int = 0):
    """Species of the pdg list (with anti-baryons added as the reference does,
    src/readindata.cpp:1033-1100): arrays of pid, mass, degeneracy, B, S, Q."""
    name = {2: "pdg-SMASH.dat", 1: "pdg-urqmd_v3.3+.dat"}.get(afterburner, "pdg-s95pv1.dat")
    rows = []
    with open(os.path.join(table_dir, name)) as f:
        lines = f.read().split("\n")
    i = 0
    while i < len(lines):
        tok = lines[i].split()
        if len(tok) < 12:
            i += 1
            continue
        pid, mass, g, B, S, Q, ndec = int(tok[0]), float(tok[2]), int(tok[4]), int(tok[5]), int(tok[6]), int(tok[10]), int(tok[11])
        rows.append((pid, mass, g, B, S, Q))
        if B > 0:
            rows.append((-pid, mass, g, -B, -S, -Q))
        i += 1 + ndec
    a = np.array(rows, dtype=np.float64)
    return {"pid": a[:, 0].astype(np.int64), "mass": a[:, 1], "g": a[:, 2],
            "B": a[:, 3], "S": a[:, 4], "Q": a[:, 5]}


def hrg_thermo(T, muB, species, nmax: int = 10):
    """Energy density, pressure (GeV/fm^3) and net-baryon density (1/fm^3) of
    an ideal hadron-resonance gas with quantum statistics (Bessel series)."""
    from scipy.special import kn
    T = np.atleast_1d(np.asarray(T, dtype=np.float64))
    muB = np.broadcast_to(np.asarray(muB, dtype=np.float64), T.shape)
    e = np.zeros_like(T)
    P = np.zeros_like(T)
    nB = np.zeros_like(T)
    keep = species["pid"] != 22
    for m, g, B in zip(species["mass"][keep], species["g"][keep], species["B"][keep]):
        if m <= 0:
            continue
        sign = 1.0 if B != 0 else -1.0   # +1 fermion, -1 boson
        lam = np.exp(B * muB / T)
        for n in range(1, (nmax if m < 0.7 else 3) + 1):
            theta = (-sign) ** (n - 1)
            x = n * m / T
            k2 = kn(2, x)
            k1 = kn(1, x)
            fug = lam ** n
            pref = g / (2.0 * np.pi ** 2) / HBARC ** 3
            P += pref * theta * fug * m * m * T * T * k2 / n ** 2
            nn = pref * theta * fug * m * m * T * k2 / n
            e += pref * theta * fug * (3.0 * m * m * T * T * k2 / n ** 2 + m ** 3 * T * k1 / n)
            nB += B * nn
    return e, P, nB


def _eos_s95(T):
    """e(T), P(T) from the s95p-v1 HRG table (columns e, P, s, T)."""
    tb = np.loadtxt(os.path.join(TABLE_DIR, "EOS_tables", "HRGEOS_PST-s95pv1.dat"))
    order = np.argsort(tb[:, 3])
    Tt, e, P = tb[order, 3], tb[order, 0], tb[order, 1]
    return np.interp(T, Tt, e), np.interp(T, Tt, P)


# --------------------------------------------------------------------------
# record construction

def _boost_matrix(u):
    """Lorentz boosts taking the fluid rest frame to the frame where the fluid
    moves with 4-velocity u ([n, 4], contravariant)."""
    n = u.shape[0]
    L = np.zeros((n, 4, 4))
    L[:, 0, 0] = u[:, 0]
    L[:, 0, 1:] = u[:, 1:]
    L[:, 1:, 0] = u[:, 1:]
    L[:, 1:, 1:] = np.eye(3)[None] + u[:, 1:, None] * u[:, None, 1:] / (1.0 + u[:, 0])[:, None, None]
    return L


def _records(tau, x, y, eta, da, u, e, T, muB, enthalpy_over_T, pi_mn, bulk, nB, q):
    n = tau.shape[0]
    r = np.zeros((n, 34), dtype=np.float64)
    r[:, 0], r[:, 1], r[:, 2], r[:, 3] = tau, x, y, eta
    r[:, 4:8] = da
    r[:, 8:12] = u
    r[:, 12] = e / HBARC
    r[:, 13] = T / HBARC
    r[:, 14] = muB / HBARC
    r[:, 17] = enthalpy_over_T
    idx = [(0, 0), (0, 1), (0, 2), (0, 3), (1, 1), (1, 2), (1, 3), (2, 2), (2, 3), (3, 3)]
    for k, (a, b) in enumerate(idx):
        r[:, 18 + k] = pi_mn[:, a, b] / HBARC
    r[:, 28] = bulk / HBARC
    r[:, 29] = nB
    r[:, 30:34] = q
    return r.astype(np.float32)


def ideal_boost_invariant(T: float = 0.150, tau: float = 10.0, dx: float = 0.5,
                          rmax: float = 10.0, umax: float = 0.6) -> Surface:
    """Ideal boost-invariant constant-tau surface (1,245 cells)."""
    g = np.arange(-rmax, rmax + 1e-9, dx)
    X, Y = np.meshgrid(g, g, indexing="ij")
    X, Y = X.ravel(), Y.ravel()
    R = np.hypot(X, Y)
    m = R < rmax
    X, Y, R = X[m], Y[m], R[m]
    n = X.size
    ur = umax * R / rmax
    phi = np.arctan2(Y, X)
    u = np.stack([np.sqrt(1.0 + ur ** 2), ur * np.cos(phi), ur * np.sin(phi), np.zeros(n)], 1)
    da = np.zeros((n, 4))
    da[:, 0] = dx * dx
    Tn = np.full(n, T)
    e, P = _eos_s95(Tn)
    zeros4 = np.zeros((n, 4, 4))
    rec = _records(np.full(n, tau), X, Y, np.zeros(n), da, u, e, Tn, np.zeros(n),
                   (e + P) / Tn, zeros4, np.zeros(n), np.zeros(n), np.zeros((n, 4)))
    return Surface(rec, hydro_mode=1, eos=2, bulk=0, rhob=0, diff=0)


def _viscous_geometry(rng, n_cells, n_eta, eta_max, radius, umax, spacelike_frac, max_ratio):
    per = n_cells // n_eta
    etas = np.linspace(-eta_max, eta_max, n_eta)
    eta = np.repeat(etas, per)
    extra = n_cells - eta.size
    if extra:
        eta = np.concatenate([eta, rng.choice(etas, extra)])
    n = eta.size
    rr = radius * np.sqrt(rng.random(n))
    ph = 2 * np.pi * rng.random(n)
    x, y = rr * np.cos(ph), rr * np.sin(ph)
    tau = rng.uniform(8.0, 14.0, n)
    ur = umax * rr / radius
    u = np.stack([np.sqrt(1.0 + ur ** 2), ur * np.cos(ph), ur * np.sin(ph), np.zeros(n)], 1)
    d_eta = 2.0 * eta_max / max(n_eta - 1, 1)
    da = np.zeros((n, 4))
    da[:, 0] = 0.5 * 0.5 * d_eta
    sl = rng.random(n) < spacelike_frac
    ratio = rng.uniform(0.0, max_ratio, n) * sl
    da[:, 1] = ratio * da[:, 0] * np.cos(ph)
    da[:, 2] = ratio * da[:, 0] * np.sin(ph)
    return tau, x, y, eta, u, da


def _shear(rng, u, enthalpy, max_ratio):
    n = u.shape[0]
    a = rng.standard_normal((n, 5))
    A = np.zeros((n, 4, 4))
    A[:, 1, 1], A[:, 2, 2] = a[:, 0], a[:, 1]
    A[:, 3, 3] = -a[:, 0] - a[:, 1]
    A[:, 1, 2] = A[:, 2, 1] = a[:, 2]
    A[:, 1, 3] = A[:, 3, 1] = a[:, 3]
    A[:, 2, 3] = A[:, 3, 2] = a[:, 4]
    norm = np.sqrt(np.einsum("nij,nij->n", A, A))
    A *= (rng.uniform(0.0, max_ratio, n) * enthalpy / norm)[:, None, None]
    L = _boost_matrix(u)
    return np.einsum("nai,nij,nbj->nab", L, A, L)


def viscous_3d(n_cells: int = 200_000, seed: int = 2, n_eta: int = 64, eta_max: float = 4.0,
               radius: float = 10.0, umax: float = 0.75) -> Surface:
    """Viscous 3+1D surface with shear, bulk and spacelike cells."""
    rng = np.random.default_rng(seed)
    tau, x, y, eta, u, da = _viscous_geometry(rng, n_cells, n_eta, eta_max, radius, umax, 0.2, 1.5)
    n = tau.size
    T = rng.uniform(0.145, 0.155, n)
    e, P = _eos_s95(T)
    w = e + P
    pi_mn = _shear(rng, u, w, 0.3)
    bulk = rng.uniform(-0.1, 0.0, n) * w
    rec = _records(tau, x, y, eta, da, u, e, T, np.zeros(n), w / T, pi_mn, bulk,
                   np.zeros(n), np.zeros((n, 4)))
    return Surface(rec, hydro_mode=2, eos=2, bulk=1, rhob=0, diff=0)


def finite_density_3d(n_cells: int = 1_000_000, seed: int = 3, n_eta: int = 64,
                      eta_max: float = 4.0, radius: float = 10.0, umax: float = 0.75,
                      table_dir: str = TABLE_DIR) -> Surface:
    """3+1D surface at finite baryon density with baryon diffusion."""
    rng = np.random.default_rng(seed)
    tau, x, y, eta, u, da = _viscous_geometry(rng, n_cells, n_eta, eta_max, radius, umax, 0.2, 1.5)
    n = tau.size
    T = rng.uniform(0.130, 0.155, n)
    muB = rng.uniform(0.0, 0.4, n)
    species = load_species(table_dir, afterburner=2)
    Tg = np.linspace(0.129, 0.156, 28)
    mg = np.linspace(0.0, 0.401, 42)
    TT, MM = np.meshgrid(Tg, mg, indexing="ij")
    eg, Pg, nBg = (v.reshape(TT.shape) for v in hrg_thermo(TT.ravel(), MM.ravel(), species))
    from scipy.interpolate import RegularGridInterpolator
    pts = np.stack([T, muB], 1)
    e = RegularGridInterpolator((Tg, mg), eg)(pts)
    P = RegularGridInterpolator((Tg, mg), Pg)(pts)
    nB = RegularGridInterpolator((Tg, mg), nBg)(pts)
    w = e + P
    pi_mn = _shear(rng, u, w, 0.3)
    bulk = rng.uniform(-0.1, 0.0, n) * w
    qdir = rng.standard_normal((n, 3))
    qdir /= np.linalg.norm(qdir, axis=1, keepdims=True)
    q_lrf = np.zeros((n, 4))
    q_lrf[:, 1:] = qdir * (rng.uniform(0.0, 0.2, n) * nB)[:, None]
    q = np.einsum("nab,nb->na", _boost_matrix(u), q_lrf)
    rec = _records(tau, x, y, eta, da, u, e, T, muB, w / T, pi_mn, bulk, nB, q)
    return Surface(rec, hydro_mode=2, eos=10, bulk=1, rhob=1, diff=1)


# --------------------------------------------------------------------------
# reader semantics and files

def music_to_fo_surf(records: np.ndarray, hydro_mode: int) -> np.ndarray:
    """FO_surf records (float32 [n, 34]) from binary MUSIC records, with the
    unit conversions and float rounding of read_FOsurfdat_MUSIC(_boost_invariant)
    (src/readindata.cpp:425-462, 652-689) and the T > 0.01 GeV filter
    (src/readindata.cpp:751-761)."""
    a = np.asarray(records, dtype=np.float32)
    f64 = a.astype(np.float64)
    out = np.zeros((a.shape[0], 34), dtype=np.float32)
    out[:, 0:3] = a[:, 0:3]
    if hydro_mode == 2:
        out[:, 3] = a[:, 3]
        out[:, 4:8] = a[:, 4:8]
    else:
        out[:, 3] = 0.0
        out[:, 4:7] = a[:, 4:7]
        out[:, 7] = 0.0
    out[:, 8:12] = a[:, 8:12]
    E = (f64[:, 12] * HBARC).astype(np.float32)
    T = (f64[:, 13] * HBARC).astype(np.float32)
    out[:, 12] = E
    out[:, 13] = T
    out[:, 14] = (a[:, 17] * T - E).astype(np.float32)        # float arithmetic
    out[:, 15] = a[:, 29]
    out[:, 16] = (f64[:, 14] * HBARC).astype(np.float32)
    out[:, 17] = (f64[:, 15] * HBARC).astype(np.float32)
    out[:, 18] = (f64[:, 16] * HBARC).astype(np.float32)
    out[:, 19:29] = (f64[:, 18:28] * HBARC).astype(np.float32)
    out[:, 29] = (f64[:, 28] * HBARC).astype(np.float32)
    out[:, 30:34] = a[:, 30:34]
    return out[T > 0.01]


def write_music_binary(path: str, records: np.ndarray) -> None:
    np.ascontiguousarray(records, dtype="<f4").tofile(path)


def write_music_input(work_dir: str, surface: Surface, binary: bool = True) -> None:
    with open(os.path.join(work_dir, "music_input"), "w") as f:
        f.write(f"EOS_to_use {surface.eos}\n")
        f.write(f"Include_Bulk_Visc_Yes_1_No_0 {surface.bulk}\n")
        f.write(f"Include_Rhob_Yes_1_No_0 {surface.rhob}\n")
        f.write(f"turn_on_baryon_diffusion {surface.diff}\n")
        f.write(f"freeze_surface_in_binary {1 if binary else 0}\n")
        f.write("EndOfData\n")


DEFAULT_PARAMETERS = {
    "hydro_mode": 2, "afterburner_type": 0, "turn_on_bulk": 0, "turn_on_rhob": 0,
    "turn_on_diff": 0, "include_deltaf_shear": 1, "include_deltaf_bulk": 0,
    "include_deltaf_diffusion": 0, "bulk_deltaf_kind": 11, "restrict_deltaf": 1,
    "deltaf_max_ratio": 1.0, "quantum_statistics": 1, "output_samples_into_files": 0,
    "store_samples_in_memory": 1, "use_OSCAR_format": 0, "use_gzip_format": 0,
    "use_binary_format": 0, "perform_decays": 0, "perform_checks": 0,
    "include_spectators": 0, "local_charge_conservation": 0, "calculate_vn": 0,
    "MC_sampling": 4, "dN_dy_sampling_model": 30, "dN_dy_sampling_para1": 0.16,
    "y_LB": -5.0, "y_RB": 5.0, "eta_s_LB": -0.5, "eta_s_RB": 0.5,
    "grouping_particles": 1, "grouping_tolerance": 0.01,
    "sample_upto_desired_particle_number": 0, "number_of_particles_needed": 100000,
    "number_of_repeated_sampling": 100, "maximum_sampling_events": 10000,
    "randomSeed": 1,
}


def write_parameters(path: str, **overrides) -> None:
    """An iSS_parameters.dat-style file ("key = value" lines)."""
    p = dict(DEFAULT_PARAMETERS)
    p.update(overrides)
    with open(path, "w") as f:
        for k, v in p.items():
            f.write(f"{k} = {v}\n")
