"""Synthetic systems: seeded sequences, random-coil starts and the five
benchmark workloads of this engine.

The random coil follows the stated benchmark recipe: bond length 5.9 A, bond
angle uniform in [90, 150] degrees, dihedral uniform in [-pi, pi), no
non-bonded pair (|i-j| >= 3) closer than 4 A.  Chains are grown bead by bead
(natural extension reference frame placement); a rejected bead is redrawn,
and after repeated failures the chain backs off a few beads.
"""
from __future__ import annotations

import math
from typing import List

import numpy as np

from .model import Chain, ForceField, Instance, Options, System

AVOGADRO = 6.02214076e23


def random_sequence(rng: np.random.Generator, n: int) -> np.ndarray:
    return rng.integers(0, 4, size=n).astype(np.int32)


def _place(a, b, c, bond, theta, phi):
    bc = c - b
    bc /= np.linalg.norm(bc)
    nrm = np.cross(b - a, bc)
    nn = np.linalg.norm(nrm)
    if nn < 1e-9:
        nrm = np.cross(bc, np.array([0.0, 0.0, 1.0]))
        if np.linalg.norm(nrm) < 1e-9:
            nrm = np.cross(bc, np.array([0.0, 1.0, 0.0]))
        nn = np.linalg.norm(nrm)
    nrm /= nn
    m = np.cross(nrm, bc)
    d2 = np.array([-bond * math.cos(theta), bond * math.sin(theta) * math.cos(phi), bond * math.sin(theta) * math.sin(phi)])
    return c + d2[0] * bc + d2[1] * m + d2[2] * nrm


def random_coil(rng: np.random.Generator, n: int, bond: float = 5.9, amin_deg: float = 90.0, amax_deg: float = 150.0,
                rmin: float = 4.0, max_tries: int = 50) -> np.ndarray:
    x = np.zeros((n, 3))
    if n == 1:
        return x
    x[1] = [bond, 0.0, 0.0]
    i = 2
    fails = 0
    while i < n:
        ok = False
        for _ in range(max_tries):
            th = math.radians(rng.uniform(amin_deg, amax_deg))
            if i == 2:
                a = x[0] + np.array([0.0, 1.0, 0.0])
                ph = rng.uniform(-math.pi, math.pi)
                p = _place(a, x[0], x[1], bond, th, ph)
            else:
                ph = rng.uniform(-math.pi, math.pi)
                p = _place(x[i - 3], x[i - 2], x[i - 1], bond, th, ph)
            if i >= 3:
                d2 = np.sum((x[: i - 2] - p) ** 2, axis=1)
                if np.any(d2 < rmin * rmin):
                    continue
            x[i] = p
            ok = True
            break
        if ok:
            i += 1
            fails = 0
        else:
            fails += 1
            i = max(2, i - min(5, 2 * fails))
    return x


def _random_rotation(rng) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def box_for_concentration(n_beads: int, molar: float) -> float:
    """Cubic box edge (A) holding n_beads at `molar` nucleotide concentration."""
    return (n_beads / (molar * AVOGADRO * 1e-27)) ** (1.0 / 3.0)


def place_chains(rng, coils: List[np.ndarray], L: float, rmin: float = 4.0) -> List[np.ndarray]:
    """Random rigid placement in a periodic cubic box without inter-chain pairs < rmin."""
    from scipy.spatial import cKDTree

    placed: List[np.ndarray] = []
    pts = np.zeros((0, 3))
    for c in coils:
        c0 = c - c.mean(axis=0)
        for _ in range(1000):
            y = c0 @ _random_rotation(rng).T + rng.uniform(0.0, L, size=3)
            if len(pts):
                tree = cKDTree(np.mod(pts, L), boxsize=L)
                d, _ = tree.query(np.mod(y, L), k=1, distance_upper_bound=rmin)
                if np.any(np.isfinite(d)):
                    continue
            placed.append(y)
            pts = np.vstack([pts, y])
            break
        else:
            raise RuntimeError("could not place chain without overlap")
    return placed


def sis_options(**kw) -> Options:
    """[Basepair] model 1, min_loop 3, no MC; [Electrostatic] cutoff 50 A type 1;
    [MD] GJF-2GJ dt 0.05, viscosity 1e-5 Pa s, margin 10 A."""
    o = Options(bp_model=1, bp_min_loop=3, flg_ele=True, ele_cutoff_type=1, ele_cutoff=50.0,
                length_per_charge=4.38178046, dt=0.05, viscosity_Pas=1e-5, nl_margin=10.0)
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def single_chain(ff: ForceField, n: int = 64, seed: int = 1001, tempK: float = 300.0, salt: float = 0.15) -> System:
    """64-nt chain, 300 K, 150 mM, no PBC."""
    rng = np.random.default_rng(seed)
    seq = random_sequence(rng, n)
    inst = Instance([Chain(seq)], tempK=tempK, ionic_strength=salt, xyz=random_coil(rng, n))
    return System(ff, sis_options(), [inst])


def crowded_box(ff: ForceField, n_chains: int = 200, n: int = 500, molar: float = 0.01, seed: int = 1002,
                tempK: float = 300.0, salt: float = 0.15, rmin: float = 10.0) -> System:
    """n_chains x n nt in a cubic PBC box at `molar` nucleotide concentration.

    Non-bonded pairs (|i-j| >= 3 in a chain, every pair between chains) start
    at least rmin apart.  The default is the WCA sigma (10 A), so the start
    carries no WCA overlap and any engine can step it without a force-capped
    relaxation; rmin = 4 gives the coil recipe's closer contacts."""
    rng = np.random.default_rng(seed)
    L = box_for_concentration(n_chains * n, molar)
    chains = [Chain(random_sequence(rng, n)) for _ in range(n_chains)]
    coils = [random_coil(rng, n, rmin=rmin) for _ in range(n_chains)]
    xyz = np.concatenate(place_chains(rng, coils, L, rmin=rmin))
    inst = Instance(chains, tempK=tempK, ionic_strength=salt, box=(L, L, L), xyz=xyz)
    return System(ff, sis_options(), [inst])


def remd_batch(ff: ForceField, n_rep: int = 64, n: int = 120, tmin: float = 280.0, tmax: float = 360.0, seed: int = 1003,
               salt: float = 0.15) -> System:
    """n_rep replicas of one sequence at geometric temperatures."""
    rng = np.random.default_rng(seed)
    seq = random_sequence(rng, n)
    xyz = random_coil(rng, n)
    temps = [tmin * (tmax / tmin) ** (k / max(1, n_rep - 1)) for k in range(n_rep)]
    insts = [Instance([Chain(seq.copy())], tempK=t, ionic_strength=salt, xyz=xyz.copy()) for t in temps]
    return System(ff, sis_options(), insts)


def uneven_batch(ff: ForceField, n_inst: int = 256, lmin: int = 20, lmax: int = 500, seed: int = 1004) -> System:
    """Independent chains: lengths U[lmin,lmax], salt U[20,500] mM, T U[280,340] K."""
    rng = np.random.default_rng(seed)
    insts = []
    for _ in range(n_inst):
        n = int(rng.integers(lmin, lmax + 1))
        seq = random_sequence(rng, n)
        salt = float(rng.uniform(0.02, 0.5))
        T = float(rng.uniform(280.0, 340.0))
        insts.append(Instance([Chain(seq)], tempK=T, ionic_strength=salt, xyz=random_coil(rng, n)))
    return System(ff, sis_options(), insts)
