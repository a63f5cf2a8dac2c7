"""Shared builders for the tests: the golden CAG47 system and small systems."""
from pathlib import Path

import numpy as np

from sis_gb300.model import Chain, ForceField, Instance, Options, System

GOLDEN = Path(__file__).resolve().parent / "golden"


def cag47_ff() -> ForceField:
    """para/rna_NHT22.ff values of the reference's CAG47 test (no dihedral)."""
    bp = dict(U0=-5.0, bond_k=3.0, bond_r=13.8, angl_k1=1.5, angl_k2=1.5, angl_k3=1.5, angl_k4=1.5, angl_theta1=1.8326,
              angl_theta2=0.9425, angl_theta3=1.8326, angl_theta4=0.9425, dihd_k1=0.5, dihd_k2=0.5, dihd_phi1=1.8326,
              dihd_phi2=1.1345)
    return ForceField(bond_k=15.0, bond_r0=5.9, angl_k=10.0, angl_t0=2.618, dih_type=0, wca_sigma=10.0, wca_eps=2.0,
                      bp_cutoff_energy=0.001, bp={k: dict(bp) for k in ("GC", "AU", "GU")})


def cag47_system(frame: int = 0) -> System:
    z = np.load(GOLDEN / "cag47.npz")
    inst = Instance([Chain.from_string(str(z["seq"]))], tempK=295.15, ionic_strength=0.15,
                    xyz=z["xyz"][frame].astype(np.float64))
    return System(cag47_ff(), Options(bp_model=1, ele_cutoff=50.0), [inst])


def pbc_md_system(ff, frame: int = 0) -> System:
    """564 beads (4 x CAG47) in the PBC box of check/test_md.dcd."""
    z = np.load(GOLDEN / "test_md.npz")
    cag = str(np.load(GOLDEN / "cag47.npz")["seq"])
    chains = [Chain.from_string(cag) for _ in range(4)]
    inst = Instance(chains, tempK=300.0, ionic_strength=0.15, box=tuple(z["box"][frame]),
                    xyz=z["xyz"][frame].astype(np.float64))
    return System(ff, Options(bp_model=1, ele_cutoff=50.0), [inst])


def t2s2hp_system(ff) -> System:
    """check/input_T2S2HP.toml: model 5, ReB angle, exponential dihedral, DH type 2."""
    z = np.load(GOLDEN / "t2s2hp.npz")
    inst = Instance([Chain.from_string(str(z["seq"]))], tempK=300.0, ionic_strength=0.15, xyz=z["xyz"].astype(np.float64))
    o = Options(bp_model=5, bp_min_loop=3, ele_cutoff_type=2, ele_cutoff=10.0)
    return System(ff, o, [inst])


def rms_rel(a, b):
    """norm-wise error: rms over beads of |a-b| divided by the rms of |b|"""
    num = np.sqrt(np.mean(np.sum((a - b) ** 2, axis=1)))
    den = np.sqrt(np.mean(np.sum(b ** 2, axis=1)))
    return num / max(den, 1e-300)


def max_rel(a, b):
    """per-bead |a-b| / max(|b|, rms|b|), maximum over beads"""
    rms = np.sqrt(np.mean(np.sum(b ** 2, axis=1)))
    d = np.sqrt(np.sum((a - b) ** 2, axis=1)) / np.maximum(np.sqrt(np.sum(b ** 2, axis=1)), rms)
    return float(d.max())
