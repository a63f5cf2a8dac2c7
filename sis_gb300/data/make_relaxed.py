"""Writes crowded_relaxed.npz: the relaxed start of the crowded-box workload.

The crowded box (200 chains x 500 nt, cubic PBC box at 10 mM nucleotide,
150 mM salt, 300 K, sequences and random-coil starts from seed 1002) starts
far from equilibrium: its coil angles are strained and its velocities are
zero.  Every timed arm of the benchmark (the GPU path, its CPU baseline and
the reference arm) starts from the same relaxed positions instead, so that
all of them see the same state, the same list rebuild rate and the same
pair-list lengths.  The relaxation is 3000 force-capped (1000 kcal/mol/A)
and 3000 free GJF-2GJ steps of the mixed path, from velocities drawn at
300 K; the positions are stored in FP32 (they are the start, not a result).

Needs a CUDA GPU:  python sis_gb300/data/make_relaxed.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
OUT = HERE / "crowded_relaxed.npz"


def main():
    sys.path.insert(0, str(ROOT))
    from sis_gb300 import MIXED
    from sis_gb300.coil import crowded_box
    from sis_gb300.engine import Engine
    from sis_gb300.inputs import read_ff

    ff = read_ff(HERE / "sis.ff")
    sysm = crowded_box(ff, 200, 500, 0.01, seed=1002)
    eng = Engine(sysm, precision=MIXED, seed=2024)
    eng.init_velocities()
    eng.relax(capped_steps=3000, fmax=1000.0, free_steps=3000)
    x, _, _ = eng.get_state(-1)
    eng.close()
    np.savez_compressed(OUT, xyz=x.astype(np.float32), seed=1002, relax_steps=np.array([3000, 3000]))
    print(OUT, x.shape)


if __name__ == "__main__":
    main()
