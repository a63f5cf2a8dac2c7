"""Output files of an MD run in the reference's formats.

* ``.out`` -- one line of energies per saved frame (write_out.F90): the
  header of ``write_out_header`` and the Fortran edit descriptors
  ``(i12, 1x, [i4, 1x,] f6.2, 7(1x, g13.6))`` plus ``(1x, g13.6)`` for Eele,
  restated here (``fortran_g``, ``fortran_e``, ``fortran_f``) from the
  Fortran standard's rules for G, E and F editing.
* ``.bp`` / ``.bpall`` -- unformatted stream (write_bp.F90,
  init_out_files.F90:103-119): the kinds (int32 2, int32 4), then per frame
  (int16 i, int16 j, float32 energy) for every formed pair (energy <= -kT
  for ``.bp``, all formed pairs for ``.bpall``) and a (0, 0, 0.0) record.
* ``.bpe`` -- per frame one line of ``(1x, i5, 1x, i5, 1x, f6.2)`` entries.
* ``.rep`` -- the replica labels at every saved exchange step; ``.twz`` --
  the force-ramp traps at every save step.
* ``.rst`` -- unformatted stream of blocks (write_rst.F90): block id
  (int32), block size in bytes (int32), payload.  Blocks STEP (int32 1,
  int64 step), XYZ/VELO/ACCEL (int32 replica, int32 nmp, nmp x 3 float64),
  REPLICA (int32 n, then n pairs of int32 replica, label) and PBC (3 float64)
  are written as the reference writes them.  The noise state is not an MT
  stream here but a Philox key and counter, which the stored key (block
  RST_NOISE) and the step number determine, so no PRNG block is written; the
  reference's reader (read_rst.F90) skips blocks it does not want by their
  size.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

# const_phys.F90: BOLTZ_KCAL_MOL = BOLTZ_J * JOUL2KCAL_MOL
BOLTZ_KCAL_MOL = 1.380649e-23 * ((1.0 / 4184.0) * 6.02214076e23)
# const_idx.F90 ENE
ENE_TOTAL, ENE_BOND, ENE_ANGL, ENE_DIHE, ENE_BP, ENE_EXV, ENE_ELE = 0, 1, 2, 3, 4, 5, 6
ENE_STAGE, ENE_TWZ, ENE_RG, ENE_REST = 7, 8, 9, 10
# const_idx.F90 RSTBLK
RST_STEP, RST_ANNEAL, RST_XYZ, RST_VELO, RST_ACCEL, RST_REPLICA, RST_PRNG, RST_PRNGREP, RST_TWZ, RST_PBC = range(1, 11)
# the noise key of the engine (Philox key and stream); not a block id of
# const_idx.F90 RSTBLK, so the reference's reader skips it by its size
RST_NOISE = 101
# var_io.F90 KIND_OUT_BP, KIND_OUT_BPE
KIND_OUT_BP, KIND_OUT_BPE = 2, 4


# ------------------------------------------------------- Fortran editing
def _stars(w: int) -> str:
    return "*" * w


def fortran_f(x: float, w: int, d: int) -> str:
    """Fw.d: d digits after the point, right-justified in w (a point and no
    digits after it for d = 0); asterisks if it does not fit."""
    s = f"{x:.{d}f}"
    if d == 0:
        s += "."
    if len(s) > w:
        return _stars(w)
    return s.rjust(w)


def fortran_e(x: float, w: int, d: int) -> str:
    """Ew.d: [-]0.d1..ddE+xx (exponent without E when beyond two digits)."""
    if x == 0.0:
        digits, e10 = "0" * d, 0
    else:
        s = f"{abs(x):.{d - 1}e}"
        mant, ex = s.split("e")
        digits = mant.replace(".", "")
        e10 = int(ex) + 1
    tail = f"E{e10:+03d}" if abs(e10) <= 99 else f"{e10:+04d}"
    s = ("-" if x < 0 else "") + "0." + digits + tail
    if len(s) > w:
        return _stars(w)
    return s.rjust(w)


def fortran_g(x: float, w: int = 13, d: int = 6) -> str:
    """Gw.d of a real: the value rounded to d significant digits is s with
    10**(k-1) <= s < 10**k; for 0 <= k <= d it is written F(w-4).(d-k)
    followed by 4 blanks, otherwise Ew.d; zero is F(w-4).(d-1) and 4 blanks."""
    if not np.isfinite(x):
        return ("NaN" if x != x else ("-Infinity" if x < 0 else "Infinity")).rjust(w)[-w:]
    if x == 0.0:
        return fortran_f(0.0, w - 4, d - 1) + "    "
    k = int(f"{abs(x):.{d - 1}e}".split("e")[1]) + 1
    if 0 <= k <= d:
        return fortran_f(x, w - 4, d - k) + "    "
    return fortran_e(x, w, d)


def fortran_i(n: int, w: int) -> str:
    s = str(int(n))
    return _stars(w) if len(s) > w else s.rjust(w)


# ------------------------------------------------------------------- .out
class OutFile:
    """The .out energy file of one replica (write_out.F90)."""

    def __init__(self, path, replica: bool = False, ele: bool = True, stage: bool = False, twz: bool = False,
                 rg: bool = False, rest: bool = False):
        """The optional columns follow write_out_header: Eele, Estage,
        Etweezers, Erg and Rg, Erest, each present when its term is on."""
        self.replica, self.ele = replica, ele
        self.stage, self.twz, self.rg, self.rest = stage, twz, rg, rest
        self.f = open(path, "w")
        if replica:
            h = ("#(1)nframe   (2)R (3)T   (4)Ekin       (5)Epot       (6)Ebond     "
                 " (7)Eangl      (8)Edih       (9)Ebp        (10)Eexv     ")
            icol = 10
        else:
            h = ("#(1)nframe   (2)T   (3)Ekin       (4)Epot       (5)Ebond     "
                 " (6)Eangl      (7)Edih       (8)Ebp        (9)Eexv      ")
            icol = 9
        for on, name in ((ele, "Eele     "), (stage, "Estage   "), (twz, "Etweezers"), (rg, "Erg      "),
                         (rg, "Rg       "), (rest, "Erest    ")):
            if on:
                icol += 1
                h += f" ({icol:2d}){name}"
        self.f.write(h + "\n")

    def write(self, step: int, tempK: float, ekin: float, energies: Sequence[float], rep_label: Optional[int] = None,
              rg: float = 0.0):
        """energies: the 11-slot vector of energy_sumup (0 total ... 10);
        rg: the radius of gyration, written after Erg."""
        s = fortran_i(step, 12) + " "
        if self.replica:
            s += fortran_i(rep_label, 4) + " "
        s += fortran_f(tempK, 6, 2)
        for v in [ekin] + [energies[i] for i in range(ENE_EXV + 1)]:
            s += " " + fortran_g(float(v))
        if self.ele:
            s += " " + fortran_g(float(energies[ENE_ELE]))
        if self.stage:
            s += " " + fortran_g(float(energies[ENE_STAGE]))
        if self.twz:
            s += " " + fortran_g(float(energies[ENE_TWZ]))
        if self.rg:
            s += " " + fortran_g(float(energies[ENE_RG])) + " " + fortran_g(float(rg))
        if self.rest:
            s += " " + fortran_g(float(energies[ENE_REST]))
        self.f.write(s + "\n")

    def close(self):
        self.f.close()


def read_out(path) -> Dict[str, np.ndarray]:
    """Columns of a .out file by their header names (nframe, T, Ekin, ...)."""
    with open(path) as f:
        head = f.readline().split()
        rows = [line.split() for line in f if line.strip()]
    names = [h.split(")", 1)[1] for h in head]
    cols = list(zip(*rows)) if rows else [[] for _ in names]
    return {n: np.array([float(v) for v in c]) for n, c in zip(names, cols)}


# ------------------------------------------------------- .bp / .bpall / .bpe
def formed_pairs(records: np.ndarray, status: np.ndarray, energies: np.ndarray, tempK: float, all_formed: bool = False):
    """(i, j, energy) of every formed pair in list order: status set and, for
    .bp/.bpe, energy <= -kT (write_bp.F90:44-56)."""
    kT = tempK * BOLTZ_KCAL_MOL
    out = []
    for r, st, e in zip(np.asarray(records), np.asarray(status), np.asarray(energies)):
        if st and (all_formed or e <= -kT):
            out.append((int(r[0]), int(r[1]), float(e)))
    return out


class BpFile:
    """.bp (formed pairs with energy <= -kT) or .bpall (every formed pair)."""

    def __init__(self, path, all_formed: bool = False):
        self.all_formed = all_formed
        self.f = open(path, "wb")
        self.f.write(struct.pack("<ii", KIND_OUT_BP, KIND_OUT_BPE))

    def write_frame(self, records, status, energies, tempK: float):
        for i, j, e in formed_pairs(records, status, energies, tempK, self.all_formed):
            self.f.write(struct.pack("<hhf", i, j, e))
        self.f.write(struct.pack("<hhf", 0, 0, 0.0))

    def close(self):
        self.f.close()


def read_bp(path) -> List[List[tuple]]:
    """Frames of a .bp/.bpall file: lists of (i, j, energy).  A file cut
    inside its header or a record, or whose last frame lacks its (0, 0, 0)
    terminator, raises ValueError."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < 8:
        raise ValueError(f"{path}: truncated .bp header")
    ki, kr = struct.unpack_from("<ii", data, 0)
    if (ki, kr) != (KIND_OUT_BP, KIND_OUT_BPE):
        raise ValueError(f"{path}: unsupported kinds {ki}, {kr}")
    if (len(data) - 8) % 8:
        raise ValueError(f"{path}: truncated .bp record at byte {8 + (len(data) - 8) // 8 * 8}")
    frames, cur = [], []
    for off in range(8, len(data), 8):
        i, j, e = struct.unpack_from("<hhf", data, off)
        if i == 0:
            frames.append(cur)
            cur = []
        else:
            cur.append((i, j, e))
    if cur:
        raise ValueError(f"{path}: the last frame has no terminator")
    return frames


class BpeFile:
    """.bpe: one line per frame of (1x, i5, 1x, i5, 1x, f6.2) entries."""

    def __init__(self, path):
        self.f = open(path, "w")

    def write_frame(self, records, status, energies, tempK: float):
        s = "".join(" " + fortran_i(i, 5) + " " + fortran_i(j, 5) + " " + fortran_f(e, 6, 2)
                    for i, j, e in formed_pairs(records, status, energies, tempK))
        self.f.write(s + "\n")

    def close(self):
        self.f.close()


# ------------------------------------------------------------- .rep, .twz
class RepFile:
    """The .rep label table of a replica-exchange run (job_md.F90:515-525):
    per saved exchange step ``(i12, 1x)`` the step, then the label of every
    replica, ``(i5, 1x)`` each and ``(i5)`` for the last."""

    def __init__(self, path):
        self.f = open(path, "w")

    def write(self, step: int, rep2lab: Sequence[int]):
        labs = [int(v) for v in rep2lab]
        s = fortran_i(step, 12) + " " + "".join(fortran_i(v, 5) + " " for v in labs[:-1]) + fortran_i(labs[-1], 5)
        self.f.write(s + "\n")

    def close(self):
        self.f.close()


# const_phys.F90 JOUL2KCAL_MOL; the tweezers output divides by it x 1e-22 for pN
JOUL2KCAL_MOL = (1.0 / 4184.0) * 6.02214076e23


def pbc_vec_d(a: np.ndarray, b: np.ndarray, box: Optional[Sequence[float]]) -> np.ndarray:
    """a - b folded once into [-box/2, box/2] per axis (pbc.F90:140-165)."""
    v = np.asarray(a, dtype=np.float64) - np.asarray(b, dtype=np.float64)
    if box is None:
        return v
    box = np.asarray(box, dtype=np.float64)
    half = 0.5 * box
    return np.where(v > half, v - box, np.where(v < -half, v + box, v))


class TwzFile:
    """The .twz force-ramp record (init_out_files.F90:133-139,
    force_tweezers.F90:55-59): at every save step, for every force-ramp pair,
    ``(i13, x, i3, 6(x, g15.8))`` of the step, the pair (1-based), the trap
    distance, the bead distance, the two trap-bead distances and the two trap
    forces in pN.  The reference writes it from the force evaluation of that
    step, so the beads are the positions the step starts from and the traps
    are at that step's positions."""

    HEADER = ("#  (1)step  (2)id (3)d[traps]   (4)d[beads]   (5)d[t1-b1]   (6)d[t2-b2]   (7)f[b1]      (8)f[b2]")

    def __init__(self, path):
        self.f = open(path, "w")
        self.f.write(self.HEADER + "\n")

    def write(self, step: int, xyz: np.ndarray, fr, box: Optional[Sequence[float]] = None):
        """xyz: the instance's coordinates at the start of ``step``; fr: its
        ForceRampPair list (1-based beads, as the input files give them)."""
        for ipair, t in enumerate(fr, start=1):
            p1 = np.asarray(t.init[0], dtype=np.float64) + np.asarray(t.velo[0], dtype=np.float64) * step
            p2 = np.asarray(t.init[1], dtype=np.float64) + np.asarray(t.velo[1], dtype=np.float64) * step
            x1, x2 = xyz[t.i - 1], xyz[t.j - 1]
            v1, v2 = pbc_vec_d(p1, x1, box), pbc_vec_d(p2, x2, box)
            n1, n2 = float(np.linalg.norm(v1)), float(np.linalg.norm(v2))
            vals = [np.linalg.norm(p2 - p1), np.linalg.norm(x2 - x1), n1, n2,
                    t.k[0] * n1 / (JOUL2KCAL_MOL * 1.0e-22), t.k[1] * n2 / (JOUL2KCAL_MOL * 1.0e-22)]
            self.f.write(fortran_i(step, 13) + " " + fortran_i(ipair, 3)
                         + "".join(" " + fortran_g(float(v), 15, 8) for v in vals) + "\n")

    def close(self):
        self.f.close()


# ------------------------------------------------------------ schedules
def read_schedule(path, ncols: int) -> List[tuple]:
    """Rows of an annealing (step, tempK) or timed Rg-bias (step, k, rg0)
    schedule file, read as Fortran list-directed input does in
    read_anneal.F90 and read_timed_bias_rg.F90: each row takes the next
    ``ncols`` values, continuing onto following lines if one holds fewer,
    and the rest of its last line is skipped.  Values are separated by
    blanks or commas.  A row with a negative step, a non-positive last value
    or (for three columns) a negative k raises ValueError, as the reference
    stops there."""
    rows = []
    with open(path) as f:
        lines = f.read().splitlines()
    k = 0
    while k < len(lines):
        toks: List[str] = []
        while len(toks) < ncols and k < len(lines):
            toks += lines[k].replace(",", " ").split()
            k += 1
        if not toks:
            break
        if len(toks) < ncols:
            raise ValueError(f"{path}: incomplete row at the end of the file")
        try:
            step = int(toks[0])
            vals = [float(t) for t in toks[1:ncols]]
        except ValueError as e:
            raise ValueError(f"{path}: cannot read row {len(rows) + 1}: {e}") from None
        if step < 0 or vals[-1] <= 0.0 or (ncols == 3 and vals[0] < 0.0):
            raise ValueError(f"{path}: invalid row {len(rows) + 1}: {' '.join(toks[:ncols])}")
        rows.append((step, *vals))
    return rows


# ------------------------------------------------------------------- .rst
@dataclass
class Restart:
    step: int = 0
    xyz: Dict[int, np.ndarray] = field(default_factory=dict)  # by replica (1-based)
    velos: Dict[int, np.ndarray] = field(default_factory=dict)
    accels: Dict[int, np.ndarray] = field(default_factory=dict)
    rep2lab: Optional[List[int]] = None
    box: Optional[np.ndarray] = None
    ianneal: Optional[int] = None  # 1-based stage of the annealing schedule
    twz_init: Dict[int, np.ndarray] = field(default_factory=dict)  # by replica: force-ramp traps at step 0, (n, 2, 3)
    noise: Dict[int, tuple] = field(default_factory=dict)  # by replica: (Philox key, stream)


def write_rst(path, step: int, xyz: np.ndarray, velos: np.ndarray, accels: np.ndarray, grep: int = 1,
              box: Optional[Sequence[float]] = None, rep2lab: Optional[Sequence[int]] = None,
              ianneal: Optional[int] = None, twz_init: Optional[np.ndarray] = None,
              noise: Optional[Tuple[int, int]] = None):
    """One replica's restart file in the block order of write_rst.F90
    (replica table first in the first replica's file, then step, annealing
    stage, coordinates, velocities, accelerations, the force-ramp traps'
    starting positions (int32 replica, int32 n, n x 2 x 3 float64), PBC
    box), and last the noise key ``noise`` = (Philox key, stream) in block
    RST_NOISE (int32 replica, uint32 stream, uint64 key).  The reference keeps
    its MT19937 state in PRNG blocks instead; the step number and this key
    determine the noise here, so no PRNG block is written."""
    xyz, velos, accels = (np.ascontiguousarray(a, dtype="<f8").reshape(-1, 3) for a in (xyz, velos, accels))
    nmp = xyz.shape[0]
    if velos.shape[0] != nmp or accels.shape[0] != nmp:
        raise ValueError("xyz, velos and accels must have the same number of beads")
    with open(path, "wb") as f:
        if rep2lab is not None and len(rep2lab) > 1:
            n = len(rep2lab)
            f.write(struct.pack("<ii", RST_REPLICA, 4 * (1 + 2 * n)))
            f.write(struct.pack("<i", n))
            for i, lab in enumerate(rep2lab, start=1):
                f.write(struct.pack("<ii", i, int(lab)))
        f.write(struct.pack("<ii", RST_STEP, 4 + 8))
        f.write(struct.pack("<iq", 1, int(step)))
        if ianneal is not None:
            f.write(struct.pack("<iii", RST_ANNEAL, 4, int(ianneal)))
        for blk, arr in ((RST_XYZ, xyz), (RST_VELO, velos), (RST_ACCEL, accels)):
            f.write(struct.pack("<ii", blk, 4 * 2 + 8 * nmp * 3))
            f.write(struct.pack("<ii", int(grep), nmp))
            f.write(arr.tobytes())
        if twz_init is not None and len(twz_init) > 0:
            t = np.ascontiguousarray(twz_init, dtype="<f8").reshape(-1, 2, 3)
            f.write(struct.pack("<iiii", RST_TWZ, 4 * 2 + 8 * t.size, int(grep), t.shape[0]))
            f.write(t.tobytes())
        if box is not None:
            f.write(struct.pack("<ii", RST_PBC, 8 * 3))
            f.write(np.asarray(box, dtype="<f8").tobytes())
        if noise is not None:
            f.write(struct.pack("<iiiIQ", RST_NOISE, 16, int(grep), int(noise[1]) & 0xFFFFFFFF,
                                int(noise[0]) & 0xFFFFFFFFFFFFFFFF))


def read_rst(path) -> Restart:
    """Blocks of a restart file (read_rst.F90); unknown blocks are skipped by
    their size.  A file that ends inside a block header or payload, a block
    whose size disagrees with its contents, or one that holds no step block
    raises ValueError (the reference stops with 'cannot read the restart
    file')."""
    r = Restart()
    seen_step = False
    with open(path, "rb") as f:
        data = f.read()
    off = 0
    while off < len(data):
        if len(data) - off < 8:
            raise ValueError(f"{path}: restart file ends inside a block header at byte {off}")
        blk, size = struct.unpack_from("<ii", data, off)
        off += 8
        if size < 0 or size > len(data) - off:
            raise ValueError(f"{path}: block {blk} at byte {off - 8} claims {size} bytes, "
                             f"{len(data) - off} are left")
        payload = data[off:off + size]
        off += size
        if blk == RST_STEP:
            if size != 12:
                raise ValueError(f"{path}: step block of {size} bytes, expected 12")
            r.step = struct.unpack("<iq", payload)[1]
            seen_step = True
        elif blk == RST_ANNEAL:
            if size != 4:
                raise ValueError(f"{path}: annealing block of {size} bytes, expected 4")
            r.ianneal = struct.unpack("<i", payload)[0]
        elif blk in (RST_XYZ, RST_VELO, RST_ACCEL):
            if size < 8:
                raise ValueError(f"{path}: block {blk} of {size} bytes")
            grep, nmp = struct.unpack("<ii", payload[:8])
            if nmp < 0 or size != 8 + 24 * nmp:
                raise ValueError(f"{path}: block {blk} of replica {grep} holds {size} bytes for {nmp} beads")
            arr = np.frombuffer(payload[8:], dtype="<f8").reshape(nmp, 3).copy()
            {RST_XYZ: r.xyz, RST_VELO: r.velos, RST_ACCEL: r.accels}[blk][grep] = arr
        elif blk == RST_REPLICA:
            n = struct.unpack("<i", payload[:4])[0] if size >= 4 else -1
            if n < 0 or size != 4 + 8 * n:
                raise ValueError(f"{path}: replica block of {size} bytes for {n} replicas")
            pairs = struct.unpack(f"<{2 * n}i", payload[4:])
            r.rep2lab = [pairs[2 * k + 1] for k in range(n)]
        elif blk == RST_TWZ:
            grep, n = struct.unpack("<ii", payload[:8]) if size >= 8 else (0, -1)
            if n < 0 or size != 8 + 48 * n:
                raise ValueError(f"{path}: tweezers block of {size} bytes for {n} trap pairs")
            r.twz_init[grep] = np.frombuffer(payload[8:], dtype="<f8").reshape(n, 2, 3).copy()
        elif blk == RST_NOISE:
            if size != 16:
                raise ValueError(f"{path}: noise-key block of {size} bytes, expected 16")
            grep, stream, key = struct.unpack("<iIQ", payload)
            r.noise[grep] = (key, stream)
        elif blk == RST_PBC:
            if size != 24:
                raise ValueError(f"{path}: PBC block of {size} bytes, expected 24")
            r.box = np.frombuffer(payload, dtype="<f8").copy()
    if not seen_step:
        raise ValueError(f"{path}: no step block")
    return r


# ------------------------------------------------------- engine frames
def save_frame(eng, inst: int, step: int, out: Optional[OutFile] = None, bp: Optional[BpFile] = None,
               bpall: Optional[BpFile] = None, bpe: Optional[BpeFile] = None, tempK: Optional[float] = None,
               rep_label: Optional[int] = None):
    """The per-frame output of job_md.F90:490-507 for one instance of an
    Engine: energies (energy_sumup, energy_kinetic) to .out and the formed
    base pairs to .bp/.bpall/.bpe."""
    tK = float(eng.system.instances[inst].tempK) if tempK is None else float(tempK)
    if out is not None:
        out.write(step, tK, eng.energy_kinetic(inst), eng.energy_sumup(inst, tK), rep_label)
    if bp is not None or bpall is not None or bpe is not None:
        rec = eng.get_list(inst, 2)
        st = eng.get_bp_status(inst)
        ene = eng.get_bp_energies(inst)
        for w in (bp, bpall, bpe):
            if w is not None:
                w.write_frame(rec, st, ene, tK)


def restart_engine(eng, path, inst: int = 0, grep: int = 1, check_noise: bool = True):
    """Loads one replica's coordinates, velocities, accelerations and step
    from a restart file into instance inst of an Engine.  When the file
    holds the noise key it was written with, the engine must have the same
    key and stream, or the run would go on with other noise (the reference
    restores its MT19937 state); ``check_noise=False`` accepts a change."""
    r = read_rst(path)
    if check_noise and grep in r.noise and hasattr(eng, "seed"):
        have = (int(eng.seed) & 0xFFFFFFFFFFFFFFFF, int(eng.streams[inst]) & 0xFFFFFFFF)
        if have != tuple(r.noise[grep]):
            raise ValueError(f"{path}: written with noise key {r.noise[grep][0]} stream {r.noise[grep][1]}, the engine "
                             f"has key {have[0]} stream {have[1]}; pass check_noise=False to continue with other noise")
    n = eng.nmp(inst)
    for name, d in (("coordinates", r.xyz), ("velocities", r.velos), ("accelerations", r.accels)):
        if grep not in d:
            raise ValueError(f"{path}: no {name} of replica {grep}")
        if d[grep].shape[0] != n:
            # read_rst.F90:95-100: 'nmp is not consistent in the restart file'
            raise ValueError(f"{path}: {name} of {d[grep].shape[0]} beads, the instance has {n}")
    eng.set_state(inst, r.xyz[grep], r.velos[grep], r.accels[grep])
    eng.set_step(r.step)
    return r
