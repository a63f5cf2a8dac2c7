"""System description of the SIS model: force field, run options, instances.

The fields mirror the reference's input files:

* :class:`ForceField` -- the ``.ff`` TOML file (``src/read_force_field.F90``);
* :class:`Options` -- ``[Basepair]``, ``[Electrostatic]`` and ``[MD]`` of the
  input TOML (``src/read_input.F90``; defaults at ``read_input.F90:398-413,
  641-679, 704-763``);
* :class:`Instance` -- one replica / independent system: chains, temperature,
  ionic strength and PBC box (``[Condition]``, ``[PBC_box]``).

Sequence codes follow ``SEQT`` in ``src/const_idx.F90``: A=0 U=1 G=2 C=3 D=4.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

SEQT = {"A": 0, "U": 1, "G": 2, "C": 3, "D": 4}
SEQ_CHARS = "AUGCD"
MOLT_LINEAR = 1
MOLT_CIRC = 2

# NNT order of src/const_idx.F90
NN_NAMES = ["GC_CG", "CC_GG", "GA_CU", "CG_GC", "AC_UG", "CA_GU", "AG_UC", "UA_AU", "AU_UA", "AA_UU",
            "GC_UG", "CU_GG", "GG_CU", "CG_GU", "AU_UG", "GA_UU", "UG_GU", "UA_GU", "GG_UU", "GU_UG", "AG_UU"]
NNEND_NAMES = ["AUonAU", "AUonCG", "AUonGU", "GUonCG", "GUonAU", "GUonGU"]
BP_FIELDS = ["U0", "bond_k", "bond_r", "angl_k1", "angl_k2", "angl_k3", "angl_k4",
             "angl_theta1", "angl_theta2", "angl_theta3", "angl_theta4",
             "dihd_k1", "dihd_k2", "dihd_phi1", "dihd_phi2"]
BP_TYPES = ["GC", "AU", "GU"]

# integrators (const_idx.F90 INTGRT)
GJF2GJ = 1
BD_EM = 2
# precision of the GPU path
FP64 = 0
MIXED = 1


@dataclass
class ForceField:
    bond_k: float = 15.0
    bond_r0: float = 5.84
    angl_reb: bool = False
    angl_k: float = 10.0
    angl_t0: float = 2.643
    dih_type: int = 1  # 0 none, 1 cosine, 2 exponential
    dih_k: float = 5.0
    dih_w: float = 0.0
    dih_p0: float = 2.861
    wca_sigma: float = 10.0
    wca_eps: float = 2.0
    bp_cutoff_energy: float = 0.001
    bp: dict = field(default_factory=dict)  # "GC"/"AU"/"GU" -> dict of BP_FIELDS
    nn_dH: List[float] = field(default_factory=lambda: [0.0] * 21)
    nn_dS: List[float] = field(default_factory=lambda: [0.0] * 21)
    dH0: float = 0.0
    dS0: float = 0.0
    coef_dG: float = 1.0
    nnend: bool = False
    nnend_dH: List[float] = field(default_factory=lambda: [0.0] * 6)
    nnend_dS: List[float] = field(default_factory=lambda: [0.0] * 6)
    dHend0: float = 0.0
    dSend0: float = 0.0

    def bp_array(self) -> np.ndarray:
        out = np.zeros((3, 15))
        for t, name in enumerate(BP_TYPES):
            d = self.bp.get(name)
            if d is None:
                continue
            out[t] = [float(d[k]) for k in BP_FIELDS]
        return out


@dataclass
class Options:
    bp_model: int = 1
    bp_min_loop: int = 3
    bp_jnext_compat: bool = False
    flg_ele: bool = True
    ele_cutoff_type: int = 1
    ele_cutoff: float = 50.0
    length_per_charge: float = 4.38178046
    ele_excl_bond: bool = True
    ele_excl_angle: bool = True
    temp_independent: int = 0
    tempK_ref: float = 0.0
    integrator: int = GJF2GJ
    dt: float = 0.05
    viscosity_Pas: float = 1e-5
    nl_margin: float = 10.0
    # [Basepair] nstep_MC, max_bp_per_nt: base-pair Monte Carlo removal every
    # nstep_bp_mc steps (0: none), at most max_bp_per_nt pairs per nucleotide
    nstep_bp_mc: int = 0
    max_bp_per_nt: int = 1


# ------------------------------------------------------- optional terms
# force.F90:62-75 (force_restraint.F90, force_tweezers.F90); bead indices
# are 1-based within the instance, as in the reference's input files.
@dataclass
class Restraint:
    """Sigmoid restraint between beads i and j (force_restraint.F90,
    energy_restraint.F90): E = -eps/2 (1 - tanh((r - d)/s)) for r < rcut.
    to_bead: the reference's Sigmoid-to-bead type, whose force acts on bead
    i only (bead j is the reference point)."""
    i: int
    j: int
    eps: float
    d: float
    s: float
    rcut: float
    to_bead: bool = False


@dataclass
class ConstantForcePair:
    """Dual-trap tweezers at constant force (force_tweezers.F90:29-36):
    +force on bead i, -force on bead j (kcal/mol/A); E = -(x_i - x_j).force."""
    i: int
    j: int
    force: Sequence[float]


@dataclass
class ForceRampPair:
    """Dual-trap tweezers with moving harmonic traps (force_tweezers.F90:38-60):
    trap t of bead (i, j)[t] sits at init[t] + velo[t] * istep, istep being the
    step taken, and pulls its bead with k[t] times the separation."""
    i: int
    j: int
    k: Sequence[float]
    init: Sequence[Sequence[float]]
    velo: Sequence[Sequence[float]]


@dataclass
class Chain:
    seq: np.ndarray  # int32 SEQT codes
    moltype: int = MOLT_LINEAR

    @staticmethod
    def from_string(s: str, moltype: int = MOLT_LINEAR) -> "Chain":
        return Chain(np.array([SEQT[c] for c in s.upper()], dtype=np.int32), moltype)

    def __len__(self) -> int:
        return int(len(self.seq))


@dataclass
class Instance:
    chains: List[Chain]
    tempK: float = 300.0
    ionic_strength: float = 0.15
    box: Optional[Sequence[float]] = None  # PBC box or None
    xyz: Optional[np.ndarray] = None  # (nmp, 3) initial coordinates
    has_charge: Optional[np.ndarray] = None

    @property
    def nmp(self) -> int:
        return int(sum(len(c) for c in self.chains))

    def seq(self) -> np.ndarray:
        return np.concatenate([c.seq for c in self.chains]).astype(np.int32)

    def charges(self) -> np.ndarray:
        if self.has_charge is not None:
            return np.asarray(self.has_charge, dtype=np.uint8)
        # init_ele.F90:63-74: all beads charged except D unless dummy_has_charge
        return (self.seq() != SEQT["D"]).astype(np.uint8)


@dataclass
class System:
    ff: ForceField
    opts: Options
    instances: List[Instance]

    @property
    def nmp(self) -> int:
        return int(sum(i.nmp for i in self.instances))

    def offsets(self) -> np.ndarray:
        return np.cumsum([0] + [i.nmp for i in self.instances])
