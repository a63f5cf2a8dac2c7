"""Energies of trajectory frames (job_dcd.F90:64-79), all frames at once.

The reference reads a DCD trajectory frame by frame and calls energy_sumup on
each.  Here every frame becomes an instance of one context (the instances
share the topology and conditions), so one set of launches builds the lists
of all frames and evaluates their energies; the 11-slot energy vectors come
back per frame.  Lists are built for every frame from its own coordinates.
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np

from .engine import Engine
from .model import FP64, Chain, ForceField, Instance, Options, System


def frame_energies(ff: ForceField, opts: Options, chains: Sequence[Chain], frames: np.ndarray, tempK: float,
                   ionic_strength: float, box: Optional[Sequence[float]] = None, precision: int = FP64) -> np.ndarray:
    """energies(0:10) of every frame (frames: (n_frames, nmp, 3)), shape (n_frames, 11)."""
    frames = np.asarray(frames, dtype=np.float64)
    insts = [Instance(list(chains), tempK=tempK, ionic_strength=ionic_strength, box=box, xyz=f) for f in frames]
    eng = Engine(System(ff, opts, insts), precision=precision)
    try:
        eng.neighbor_list(-1)
        return np.stack([eng.energy_sumup(k) for k in range(len(insts))])
    finally:
        eng.close()


def dcd_energies(path, ff: ForceField, opts: Options, chains: Sequence[Chain], tempK: float, ionic_strength: float,
                 precision: int = FP64) -> np.ndarray:
    """frame_energies of a DCD file (the box, if the file has one, sets PBC)."""
    from .dcd import read_dcd

    frames, boxes = read_dcd(path)
    box = None
    if boxes is not None and len(boxes) and boxes[0][0] > 0:
        box = tuple(float(b) for b in boxes[0])
    return frame_energies(ff, opts, chains, frames, tempK, ionic_strength, box=box, precision=precision)
