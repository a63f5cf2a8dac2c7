"""CHARMM DCD trajectories as the reference writes and reads them
(``src/dcd.F90:287-356`` header, ``:538-596`` frames).

Stream layout: 84-byte block ("CORD" + 20 control int32; control(11) = 1 when
a unit-cell record precedes each frame, control(20) = 24), a title block, the
atom count, then per frame an optional 48-byte unit cell (box x, 0, box y, 0,
0, box z as float64) and three float32 coordinate blocks, each framed by its
int32 byte size.
"""
from __future__ import annotations

import struct
from typing import List, Optional, Tuple

import numpy as np


def write_header(f, natom: int, unitcell: bool) -> None:
    control = [0] * 20
    control[10] = 1 if unitcell else 0
    control[19] = 24
    f.write(struct.pack("<i", 84) + b"CORD" + struct.pack("<20i", *control) + struct.pack("<i", 84))
    f.write(struct.pack("<ii", 84, 1) + b" " * 80 + struct.pack("<i", 84))
    f.write(struct.pack("<iii", 4, natom, 4))


def write_frame(f, xyz: np.ndarray, box: Optional[Tuple[float, float, float]] = None,
                fix_com_origin: bool = False) -> None:
    """One frame; with fix_com_origin the coordinates are written relative to
    their centroid, summed bead by bead in FP64 (dcd.F90:576-581)."""
    xyz = np.asarray(xyz, dtype=np.float64)
    if fix_com_origin and xyz.shape[0] > 0:
        com = np.array([np.cumsum(xyz[:, k])[-1] for k in range(3)]) / float(xyz.shape[0])
        xyz = xyz - com
    if box is not None:
        f.write(struct.pack("<i", 48) + struct.pack("<6d", box[0], 0.0, box[1], 0.0, 0.0, box[2]) + struct.pack("<i", 48))
    n = xyz.shape[0]
    for k in range(3):
        f.write(struct.pack("<i", 4 * n) + xyz[:, k].astype("<f4").tobytes() + struct.pack("<i", 4 * n))


def write_dcd(path, frames: List[np.ndarray], box=None) -> None:
    with open(path, "wb") as f:
        write_header(f, frames[0].shape[0], box is not None)
        for x in frames:
            write_frame(f, x, box)


def read_dcd(path) -> Tuple[np.ndarray, Optional[np.ndarray]]:
    """Returns (frames (nframe, natom, 3) float64, boxes (nframe, 3) or None).
    The file may end only between frames; a record cut short or framed by
    unequal sizes raises ValueError (the reference's read_onestep stops
    there too)."""
    data = open(path, "rb").read()
    pos = 0

    def block():
        nonlocal pos
        if pos + 4 > len(data):
            raise ValueError(f"{path}: truncated DCD record at byte {pos}")
        (sz,) = struct.unpack_from("<i", data, pos)
        if sz < 0 or pos + 8 + sz > len(data):
            raise ValueError(f"{path}: truncated DCD record at byte {pos}")
        payload = data[pos + 4: pos + 4 + sz]
        (sz2,) = struct.unpack_from("<i", data, pos + 4 + sz)
        if sz != sz2:
            raise ValueError(f"{path}: corrupt DCD record at byte {pos}")
        pos += 8 + sz
        return payload

    hdr = block()
    if hdr[:4] != b"CORD":
        raise ValueError("not a DCD file")
    control = struct.unpack_from("<20i", hdr, 4)
    unitcell = control[10] == 1
    block()  # title
    (natom,) = struct.unpack("<i", block())
    frames, boxes = [], []
    while pos < len(data):
        if unitcell:
            uc = struct.unpack("<6d", block())
            boxes.append((uc[0], uc[2], uc[5]))
        xs = [np.frombuffer(block(), dtype="<f4") for _ in range(3)]
        if any(x.size != natom for x in xs):
            raise ValueError(f"{path}: a frame holds a coordinate block of another atom count than {natom}")
        frames.append(np.stack(xs, axis=1).astype(np.float64))
    return np.array(frames).reshape(-1, natom, 3), (np.array(boxes) if unitcell else None)
