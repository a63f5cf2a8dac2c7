"""Readers for the reference's input formats.

* ``.ff`` force-field TOML (``src/read_force_field.F90:32-372``);
* input TOML sections used by the hot path (``src/read_input.F90``);
* FASTA (``src/read_fasta.F90``), XYZ (``src/read_xyz.F90``) and PDB
  coordinate records (``src/read_pdb.F90``).

TOML parsing uses Python's ``tomllib``; the reference uses the toml-f library
(``subprojects/toml-f``, not vendored), whose key semantics are restated here.
"""
from __future__ import annotations

import tomllib
from pathlib import Path
from typing import Dict, List, Tuple

import numpy as np

from .model import (BD_EM, BP_FIELDS, GJF2GJ, NN_NAMES, NNEND_NAMES, Chain, ConstantForcePair, ForceField,
                    ForceRampPair, Options, Restraint)


class InputError(ValueError):
    """Raised where the reference calls sis_abort on an invalid input."""


def _lower_keys(d):
    if isinstance(d, dict):
        return {k.lower() if isinstance(k, str) else k: _lower_keys(v) for k, v in d.items()}
    return d


def parse_ff(text: str, bp_model: int = 1) -> ForceField:
    """Force-field file semantics of read_force_field.F90:80-372."""
    t = tomllib.loads(text)
    pot = t.get("potential")
    if pot is None:
        raise InputError("[potential] required in FF file")
    ff = ForceField()
    bond = pot.get("bond")
    if bond is None:
        raise InputError("[bond] parameters required in FF file")
    ff.bond_k, ff.bond_r0 = float(bond["k"]), float(bond["r0"])
    angle, reb = pot.get("angle"), pot.get("angle_ReB")
    if angle is not None and reb is not None:
        raise InputError("[angle] and [angle_ReB] cannot be specified together in FF file.")
    if angle is None and reb is None:
        raise InputError("Either [angle] or [angle_ReB] parameters are required in FF file")
    a = angle if angle is not None else reb
    ff.angl_reb = reb is not None
    ff.angl_k, ff.angl_t0 = float(a["k"]), float(a["a0"])
    dcos, dexp = pot.get("dihedral"), pot.get("dihedral_exp")
    ff.dih_type = 0
    if dcos is not None:
        ff.dih_type, ff.dih_k, ff.dih_p0 = 1, float(dcos["k"]), float(dcos["phi0"])
    if dexp is not None:
        ff.dih_type, ff.dih_k, ff.dih_w, ff.dih_p0 = 2, float(dexp["k"]), float(dexp["w"]), float(dexp["phi0"])
    bp = pot.get("basepair")
    if bp is None:
        raise InputError("[basepair] parameters required in FF file")
    ff.bp_cutoff_energy = float(bp.get("cutoff_energy", 0.001))
    ff.coef_dG = float(bp.get("coef_dG", 1.0))
    ff.dH0 = float(bp.get("dH0", 0.0))
    ff.dS0 = float(bp.get("dS0", 0.0))
    ff.nnend = bool(bp.get("NNend", False))
    ff.dHend0 = float(bp.get("dHend0", 0.0))
    ff.dSend0 = float(bp.get("dSend0", 0.0))
    for name in ("GC", "AU", "GU"):
        sub = bp.get(name)
        if sub is not None:
            ff.bp[name] = {k: float(sub[k]) for k in BP_FIELDS}
    wca = pot.get("wca")
    if wca is None:
        raise InputError("[wca] parameters required in FF file")
    ff.wca_sigma, ff.wca_eps = float(wca["sigma"]), float(wca["epsilon"])
    if bp_model == 5:
        nn = t.get("NN")
        if nn is None or "dH" not in nn or "dS" not in nn:
            raise InputError("[NN.dH] and [NN.dS] required in FF file")
        ff.nn_dH = [float(nn["dH"][k]) for k in NN_NAMES]
        ff.nn_dS = [float(nn["dS"][k]) for k in NN_NAMES]
        if ff.nnend:
            ne = t.get("NNend")
            if ne is None:
                raise InputError("[NNend] required in FF file")
            ff.nnend_dH = [float(ne["dH"][k]) for k in NNEND_NAMES]
            ff.nnend_dS = [float(ne["dS"][k]) for k in NNEND_NAMES]
    return ff


def read_ff(path, bp_model: int = 1) -> ForceField:
    return parse_ff(Path(path).read_text(), bp_model)


def parse_input(text: str) -> Tuple[Options, Dict]:
    """Hot-path options from an input TOML (section names are case-insensitive
    in the reference's reader).  Returns (Options, condition dict)."""
    t = _lower_keys(tomllib.loads(text))
    o = Options()
    md = t.get("md", {})
    integ = md.get("integrator", "GJF-2GJ")
    if integ == "GJF-2GJ":
        o.integrator = GJF2GJ
    elif integ == "Ermak-McCammon":
        o.integrator = BD_EM
    else:
        raise InputError(f"invalid integrator {integ!r}")
    o.dt = float(md.get("dt", o.dt))
    m = float(md.get("neighbor_list_margin", -1.0))
    o.nl_margin = 10.0 if m < 0 else m
    v = float(md.get("viscosity_pas", -1.0))
    o.viscosity_Pas = 1e-5 if v < 0 else v
    bp = t.get("basepair")
    if bp is None:
        # read_input.F90:674-679
        o.bp_model, o.bp_min_loop = 5, 3
    else:
        o.bp_model = int(bp.get("model", 1))
        o.bp_min_loop = int(bp.get("min_loop", 3))
    ele = t.get("electrostatic")
    o.flg_ele = ele is not None
    if ele is not None:
        o.ele_cutoff_type = int(ele.get("cutoff_type", 1))
        o.ele_cutoff = float(ele.get("cutoff", 50.0))
        o.length_per_charge = float(ele.get("length_per_charge", o.length_per_charge))
        o.ele_excl_bond = bool(ele.get("exclude_covalent_bond_pairs", True))
        o.ele_excl_angle = bool(ele.get("exclude_covalent_angle_pairs", True))
    cond = t.get("condition", {})
    o.temp_independent = int(cond.get("temp_independent", 0))
    o.tempK_ref = float(cond.get("tempk_ref", 0.0))
    c = {"tempK": float(cond.get("tempk", 300.0)), "rng_seed": int(cond.get("rng_seed", 0)),
         "ionic_strength": float(ele.get("ionic_strength", 0.15)) if ele else 0.15}
    pbc = t.get("pbc_box")
    if pbc is not None:
        c["box"] = [float(pbc["x"]), float(pbc["y"]), float(pbc["z"])]
    return o, c


def read_fasta(path) -> List[Chain]:
    chains: List[Chain] = []
    cur: List[str] = []
    for line in Path(path).read_text().splitlines():
        line = line.strip()
        if not line:
            continue
        if line.startswith(">"):
            if cur:
                chains.append(Chain.from_string("".join(cur)))
            cur = []
        else:
            cur.append(line)
    if cur:
        chains.append(Chain.from_string("".join(cur)))
    return chains


def read_xyz(path) -> np.ndarray:
    lines = Path(path).read_text().splitlines()
    n = int(lines[0].split()[0])
    return np.array([[float(v) for v in lines[2 + i].split()[1:4]] for i in range(n)])


def read_pdb(path) -> np.ndarray:
    xyz = []
    for line in Path(path).read_text().splitlines():
        if line.startswith(("ATOM", "HETATM")):
            xyz.append([float(line[30:38]), float(line[38:46]), float(line[46:54])])
    return np.array(xyz)


# ------------------------------------------------------- optional terms
# const_phys.F90 JOUL2KCAL_MOL: forces in pN times JOUL2KCAL_MOL x 1e-22 are
# kcal/mol/A (read_input.F90:1060)
JOUL2KCAL_MOL = (1.0 / 4184.0) * 6.02214076e23
PN_TO_KCAL_MOL_A = JOUL2KCAL_MOL * 1.0e-22


def parse_restraints(text: str) -> List[Restraint]:
    """Restraints of a restraint file (read_restraint.F90): lines starting
    with ``Sigmoid-to-bead`` or ``Sigmoid`` followed by the two bead numbers
    (1-based), epsilon, d, s and r_cut; ``#`` lines and blank lines are
    skipped, any other line is an error."""
    out: List[Restraint] = []
    for n, line in enumerate(text.splitlines(), start=1):
        if line.startswith("#") or not line.strip():
            continue
        if line.startswith("Sigmoid-to-bead"):
            rest, to_bead = line[15:], True
        elif line.startswith("Sigmoid"):
            rest, to_bead = line[7:], False
        else:
            raise InputError(f"line {n}: unknown restraint type: {line.strip()}")
        f = rest.replace(",", " ").split()
        if len(f) < 6:
            raise InputError(f"line {n}: a restraint needs two beads, epsilon, d, s and r_cut")
        try:
            i, j = int(f[0]), int(f[1])
            eps, d, s, rcut = (float(v) for v in f[2:6])
        except ValueError as e:
            raise InputError(f"line {n}: {e}") from None
        out.append(Restraint(i, j, eps, d, s, rcut, to_bead=to_bead))
    return out


def read_restraints(path) -> List[Restraint]:
    return parse_restraints(Path(path).read_text())


def constant_force_pairs(id_pairs, forces_pN) -> List[ConstantForcePair]:
    """[Tweezers.Dual_Constant_Force] id_pairs and forces_pN
    (read_input.F90:983-1063): the forces in kcal/mol/A."""
    if len(id_pairs) != len(forces_pN):
        raise InputError("forces_pN needs one vector per pair of id_pairs")
    out = []
    for (i, j), fv in zip(id_pairs, forces_pN):
        if int(i) < 1 or int(j) < 1 or len(fv) != 3:
            raise InputError("invalid id_pairs or forces_pN in [Tweezers.Dual_Constant_Force]")
        out.append(ConstantForcePair(int(i), int(j), tuple(float(v) * PN_TO_KCAL_MOL_A for v in fv)))
    return out


def force_ramp_pairs(xyz: np.ndarray, id_pairs, spring_const, trap_speed, init=None) -> List[ForceRampPair]:
    """[Tweezers.Force_Ramp] pairs with their moving traps (init_tweezers.F90):
    the traps start on the two beads (or at ``init``, the (n, 2, 3) starting
    positions a restart file holds) and move apart along the axis from the
    first trap to the second, trap 1 at -speed_1 and trap 2 at +speed_2
    (A per step)."""
    n = len(id_pairs)
    if len(spring_const) != n or len(trap_speed) != n:
        raise InputError("spring_const and trap_speed need one pair of values per pair of id_pairs")
    xyz = np.asarray(xyz, dtype=np.float64)
    out = []
    for q, ((i, j), k, sp) in enumerate(zip(id_pairs, spring_const, trap_speed)):
        i, j = int(i), int(j)
        if not (1 <= i <= len(xyz) and 1 <= j <= len(xyz)) or len(k) != 2 or len(sp) != 2:
            raise InputError("invalid id_pairs, spring_const or trap_speed in [Tweezers.Force_Ramp]")
        p = (np.array([xyz[i - 1], xyz[j - 1]]) if init is None
             else np.asarray(init, dtype=np.float64).reshape(-1, 2, 3)[q])
        v = p[1] - p[0]
        u = v / np.sqrt(np.dot(v, v))
        velo = (tuple(-u * float(sp[0])), tuple(u * float(sp[1])))
        out.append(ForceRampPair(i, j, (float(k[0]), float(k[1])), (tuple(p[0]), tuple(p[1])), velo))
    return out


# ------------------------------------------------------- secondary structure
# [Files.In] ct / bpseq / bpl (read_ss.F90): the base pairs that the
# base-pair term may form.  The readers return (imp, jmp) pairs, 1-based
# nucleotide numbers over all chains of an instance, as the files give them.
def parse_ct(text: str, nmp: int) -> List[Tuple[int, int]]:
    """CT: a header line whose first field is the nucleotide count, then one
    line per nucleotide: index, base, prev, next, partner (0: none), index."""
    lines = [l for l in text.splitlines() if l.strip()]
    if not lines or int(lines[0].split()[0]) != nmp:
        raise ValueError("CT file: the total number of nucleotides does not match")
    out = []
    for l, line in enumerate(lines[1:nmp + 1], start=1):
        f = line.split()
        if len(f) < 6 or int(f[0]) != l:
            raise ValueError(f"CT file: line of nucleotide {l} cannot be read")
        if int(f[4]) != 0:
            out.append((l, int(f[4])))
    if len(lines) < nmp + 1:
        raise ValueError("CT file: fewer lines than nucleotides")
    return out


def parse_bpseq(text: str, nmp: int) -> List[Tuple[int, int]]:
    """BPSEQ: one line per nucleotide: index, base, partner (0: none)."""
    lines = [l for l in text.splitlines() if l.strip()]
    if len(lines) < nmp:
        raise ValueError("BPSEQ file: fewer lines than nucleotides")
    out = []
    for l, line in enumerate(lines[:nmp], start=1):
        f = line.split()
        if len(f) < 3 or int(f[0]) != l:
            raise ValueError(f"BPSEQ file: line of nucleotide {l} cannot be read")
        if int(f[2]) != 0:
            out.append((l, int(f[2])))
    return out


def parse_bpl(text: str) -> List[Tuple[int, int]]:
    """BPL: one pair per line: imp, jmp."""
    out = []
    for k, line in enumerate(l for l in text.splitlines() if l.strip()):
        f = line.split()
        if len(f) < 2:
            raise ValueError(f"BPL file: line {k + 1} cannot be read")
        out.append((int(f[0]), int(f[1])))
    return out


def read_ss(path, nmp: int) -> List[Tuple[int, int]]:
    """The pairs of a .ct, .bpseq or .bpl file (by its suffix)."""
    path = Path(path)
    text = path.read_text()
    suf = path.suffix.lower()
    if suf == ".ct":
        return parse_ct(text, nmp)
    if suf == ".bpseq":
        return parse_bpseq(text, nmp)
    if suf == ".bpl":
        return parse_bpl(text)
    raise ValueError(f"{path}: expected a .ct, .bpseq or .bpl file")


def filter_ss_pairs(inst, pairs, bp_model: int, bp_min_loop: int = 3):
    """read_ss.F90's checks of every listed pair: a chain end (i or j first
    or last of its chain), a loop shorter than the minimum, an isolated pair
    (models 3-5: neither i-1/j+1 nor i+1/j-1 complementary), or a pair of no
    known type (GC CG AU UA GU UG) is dropped with a warning.  Returns the
    kept pairs (imp < jmp, 1-based) and the warnings."""
    comp = {(0, 1), (1, 0), (1, 2), (2, 3), (2, 1), (3, 2)}  # const_idx.F90 is_complement
    canon = {(2, 3), (3, 2), (0, 1), (1, 0), (2, 1), (1, 2)}
    seq = inst.seq()
    chain_of, local = [], []
    for c, ch in enumerate(inst.chains):
        chain_of += [c] * len(ch)
        local += list(range(1, len(ch) + 1))
    kept, warn = [], []
    for imp, jmp in pairs:
        if jmp < imp:
            imp, jmp = jmp, imp
        if not (1 <= imp <= len(seq) and 1 <= jmp <= len(seq)):
            raise ValueError(f"secondary structure pair ({imp}, {jmp}) is outside the {len(seq)} nucleotides")
        i, j = local[imp - 1], local[jmp - 1]
        ic, jc = chain_of[imp - 1], chain_of[jmp - 1]
        ni, nj = len(inst.chains[ic]), len(inst.chains[jc])
        if i == 1 or i == ni:
            warn.append(f"pair ({imp}, {jmp}) not considered: i is a chain end")
            continue
        if j == 1 or j == nj:
            warn.append(f"pair ({imp}, {jmp}) not considered: j is a chain end")
            continue
        if ic == jc and i + bp_min_loop >= j:
            warn.append(f"pair ({imp}, {jmp}) not considered: minimum loop length")
            continue
        if bp_model in (3, 4, 5) and (seq[imp - 2], seq[jmp]) not in comp and (seq[imp], seq[jmp - 2]) not in comp:
            warn.append(f"pair ({imp}, {jmp}) not considered: isolated base pair")
            continue
        if (seq[imp - 1], seq[jmp - 1]) not in canon:
            warn.append(f"pair ({imp}, {jmp}) does not form any known type of base pair")
            continue
        kept.append((imp, jmp))
    return kept, warn
