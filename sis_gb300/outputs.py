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
* ``.rst`` -- unformatted stream of blocks (write_rst.F90): block id
  (int32), block size in bytes (int32), payload.  Blocks STEP (int32 1,
  int64 step), XYZ/VELO/ACCEL (int32 replica, int32 nmp, nmp x 3 float64),
  REPLICA (int32 n, then n pairs of int32 replica, label) and PBC (3 float64)
  are written as the reference writes them.  The noise state is not an MT
  stream here but the Philox counter, which the step number determines, so
  no PRNG block is written; the reference's reader (read_rst.F90) skips
  blocks by their size and needs none of them to load the rest.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np

# const_phys.F90: BOLTZ_KCAL_MOL = BOLTZ_J * JOUL2KCAL_MOL
BOLTZ_KCAL_MOL = 1.380649e-23 * ((1.0 / 4184.0) * 6.02214076e23)
# const_idx.F90 ENE
ENE_TOTAL, ENE_BOND, ENE_ANGL, ENE_DIHE, ENE_BP, ENE_EXV, ENE_ELE = 0, 1, 2, 3, 4, 5, 6
# const_idx.F90 RSTBLK
RST_STEP, RST_ANNEAL, RST_XYZ, RST_VELO, RST_ACCEL, RST_REPLICA, RST_PRNG, RST_PRNGREP, RST_TWZ, RST_PBC = range(1, 11)
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

    def __init__(self, path, replica: bool = False, ele: bool = True):
        self.replica, self.ele = replica, ele
        self.f = open(path, "w")
        if replica:
            h = ("#(1)nframe   (2)R (3)T   (4)Ekin       (5)Epot       (6)Ebond     "
                 " (7)Eangl      (8)Edih       (9)Ebp        (10)Eexv     ")
            icol = 10
        else:
            h = ("#(1)nframe   (2)T   (3)Ekin       (4)Epot       (5)Ebond     "
                 " (6)Eangl      (7)Edih       (8)Ebp        (9)Eexv      ")
            icol = 9
        if ele:
            icol += 1
            h += f" ({icol:2d})Eele     "
        self.f.write(h + "\n")

    def write(self, step: int, tempK: float, ekin: float, energies: Sequence[float], rep_label: Optional[int] = None):
        """energies: the 11-slot vector of energy_sumup (0 total ... 10)."""
        s = fortran_i(step, 12) + " "
        if self.replica:
            s += fortran_i(rep_label, 4) + " "
        s += fortran_f(tempK, 6, 2)
        for v in [ekin] + [energies[i] for i in range(ENE_EXV + 1)]:
            s += " " + fortran_g(float(v))
        if self.ele:
            s += " " + fortran_g(float(energies[ENE_ELE]))
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
    """Frames of a .bp/.bpall file: lists of (i, j, energy)."""
    with open(path, "rb") as f:
        ki, kr = struct.unpack("<ii", f.read(8))
        if (ki, kr) != (KIND_OUT_BP, KIND_OUT_BPE):
            raise ValueError(f"unsupported kinds {ki}, {kr}")
        frames, cur = [], []
        while True:
            b = f.read(8)
            if len(b) < 8:
                break
            i, j, e = struct.unpack("<hhf", b)
            if i == 0:
                frames.append(cur)
                cur = []
            else:
                cur.append((i, j, e))
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


# ------------------------------------------------------------------- .rst
@dataclass
class Restart:
    step: int = 0
    xyz: Dict[int, np.ndarray] = field(default_factory=dict)  # by replica (1-based)
    velos: Dict[int, np.ndarray] = field(default_factory=dict)
    accels: Dict[int, np.ndarray] = field(default_factory=dict)
    rep2lab: Optional[List[int]] = None
    box: Optional[np.ndarray] = None


def write_rst(path, step: int, xyz: np.ndarray, velos: np.ndarray, accels: np.ndarray, grep: int = 1,
              box: Optional[Sequence[float]] = None, rep2lab: Optional[Sequence[int]] = None):
    """One replica's restart file in the block order of write_rst.F90
    (replica table first in the first replica's file, then step, coordinates,
    velocities, accelerations, PBC box)."""
    xyz, velos, accels = (np.ascontiguousarray(a, dtype="<f8").reshape(-1, 3) for a in (xyz, velos, accels))
    nmp = xyz.shape[0]
    with open(path, "wb") as f:
        if rep2lab is not None and len(rep2lab) > 1:
            n = len(rep2lab)
            f.write(struct.pack("<ii", RST_REPLICA, 4 * (1 + 2 * n)))
            f.write(struct.pack("<i", n))
            for i, lab in enumerate(rep2lab, start=1):
                f.write(struct.pack("<ii", i, int(lab)))
        f.write(struct.pack("<ii", RST_STEP, 4 + 8))
        f.write(struct.pack("<iq", 1, int(step)))
        for blk, arr in ((RST_XYZ, xyz), (RST_VELO, velos), (RST_ACCEL, accels)):
            f.write(struct.pack("<ii", blk, 4 * 2 + 8 * nmp * 3))
            f.write(struct.pack("<ii", int(grep), nmp))
            f.write(arr.tobytes())
        if box is not None:
            f.write(struct.pack("<ii", RST_PBC, 8 * 3))
            f.write(np.asarray(box, dtype="<f8").tobytes())


def read_rst(path) -> Restart:
    """Blocks of a restart file (read_rst.F90); unknown blocks are skipped by
    their size."""
    r = Restart()
    with open(path, "rb") as f:
        while True:
            b = f.read(8)
            if len(b) < 8:
                break
            blk, size = struct.unpack("<ii", b)
            payload = f.read(size)
            if blk == RST_STEP:
                r.step = struct.unpack("<iq", payload[:12])[1]
            elif blk in (RST_XYZ, RST_VELO, RST_ACCEL):
                grep, nmp = struct.unpack("<ii", payload[:8])
                arr = np.frombuffer(payload[8:8 + 24 * nmp], dtype="<f8").reshape(nmp, 3).copy()
                {RST_XYZ: r.xyz, RST_VELO: r.velos, RST_ACCEL: r.accels}[blk][grep] = arr
            elif blk == RST_REPLICA:
                n = struct.unpack("<i", payload[:4])[0]
                pairs = struct.unpack(f"<{2 * n}i", payload[4:4 + 8 * n])
                r.rep2lab = [pairs[2 * k + 1] for k in range(n)]
            elif blk == RST_PBC:
                r.box = np.frombuffer(payload[:24], dtype="<f8").copy()
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


def restart_engine(eng, path, inst: int = 0, grep: int = 1):
    """Loads one replica's coordinates, velocities, accelerations and step
    from a restart file into instance inst of an Engine."""
    r = read_rst(path)
    eng.set_state(inst, r.xyz[grep], r.velos[grep], r.accels[grep])
    eng.set_step(r.step)
    return r
