"""Generates tests/golden/outputs.json: files written by sis_gb300.outputs
and sis_gb300.dcd for a fixed table of frames, and what the reference's own
readers (utils/sisout.py, utils/sisbp.py, utils/dcd.py of the reference
tree) make of them.

Run in a container that holds the reference tree:
    python tests/golden/make_output_fixtures.py /path/to/reference
The reference's sisbp.py imports an error class from a package that is not
part of the tree; a stand-in module with that class is installed first.
"""
import json
import sys
import tempfile
import types
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from sis_gb300 import dcd as sdcd  # noqa: E402
from sis_gb300.outputs import BpFile, OutFile  # noqa: E402

# frames: step, T, Ekin, energies[0..10]; values chosen to exercise every
# branch of G editing (F forms with 6..0 decimals, E forms, zero, negatives)
FRAMES = [
    (0, 300.0, 41.868614648997, [29.1441412318505, 0.003363370866894, 4.398169526634435, 0.0, -11.058858430180448,
                                 0.0, 35.8, 0, 0, 0, 0]),
    (100, 300.0, 1234.5678, [-0.05, 99999.9, 999999.4, 1.0e-7, -2.5e8, 0.1, -0.0999999, 0, 0, 0, 0]),
    (123456789, 310.15, 7.0, [1.0, -1.0, 12.345678, 123.4567, 1234.567, 12345.67, 123456.7, 0, 0, 0, 0]),
]
# base-pair records (i, j), status and energies of two frames at 300 K
BP_FRAMES = [
    ([(5, 20), (6, 19), (7, 18), (30, 44)], [1, 1, 0, 1], [-3.2, -0.4, -5.0, -1.5]),
    ([(5, 20), (6, 19)], [1, 1], [-0.2, -2.75]),
]
# optional-term energies (slots 7-10) for the .out columns
OPT_FRAMES = [(50, 300.0, 2.5, [float(v) for v in (-1.5, 0.5, 1.0, -2.0, 0.25, 3.0, -0.75, 0.125, 1.5, 2.25, 0.0625)],
               18.75)]
# two DCD frames of five beads, PBC box, written with fix_com_origin
DCD_FRAMES = [[[1.0 + i, 2.0 * i, -3.0 + 0.5 * i] for i in range(5)],
              [[10.25 - i, 0.125 * i * i, 7.0] for i in range(5)]]
DCD_BOX = [100.0, 110.0, 120.0]


def main(ref: Path):
    sys.path.insert(0, str(ref / "utils"))
    lop = types.ModuleType("lop")
    elements = types.ModuleType("lop.elements")
    error = types.ModuleType("lop.elements.error")

    class MyError(Exception):
        pass

    error.MyError = MyError
    sys.modules.update({"lop": lop, "lop.elements": elements, "lop.elements.error": error})
    import dcd as rdcd  # noqa: E402
    import sisbp  # noqa: E402
    import sisout  # noqa: E402

    out = {}
    with tempfile.TemporaryDirectory() as d:
        for replica in (False, True):
            p = Path(d) / f"run{int(replica)}.out"
            w = OutFile(p, replica=replica, ele=True)
            for k, (step, T, ekin, e) in enumerate(FRAMES):
                w.write(step, T, ekin, e, rep_label=k + 1 if replica else None)
            w.close()
            text = p.read_text()
            f = sisout.SisoutFile(str(p))
            f.open_to_read()
            f.read_header()
            cols = {k: v for k, v in vars(f.head_col).items() if v is not None}
            rows = []
            while f.has_more_data():
                rows.append([float(v) for v in f.read_onestep()[0][0]])
            f.close()
            out[f"out_replica{int(replica)}"] = {"text": text, "columns": cols, "rows": rows}
        p = Path(d) / "run.bp"
        w = BpFile(p)
        for pairs, st, ene in BP_FRAMES:
            w.write_frame(np.array(pairs), np.array(st), np.array(ene), 300.0)
        w.close()
        f = sisbp.SisbpFile(str(p))
        f.open_to_read()
        frames = []
        while f.has_more_data():
            pairs, energies = f.read_onestep()
            frames.append({"pairs": [list(q) for q in pairs], "energies": [float(e) for e in energies]})
        f.close()
        out["bp"] = {"bytes_hex": p.read_bytes().hex(), "frames": frames}
        p = Path(d) / "opt.out"
        # the reference's reader knows the Estage and Etweezers columns (it
        # raises on Erg, Rg and Erest)
        w = OutFile(p, ele=True, stage=True, twz=True)
        for step, T, ekin, e, rg in OPT_FRAMES:
            w.write(step, T, ekin, e, rg=rg)
        w.close()
        f = sisout.SisoutFile(str(p))
        f.open_to_read()
        f.read_header()
        cols = {k: v for k, v in vars(f.head_col).items() if v is not None}
        rows = []
        while f.has_more_data():
            rows.append([float(v) for v in f.read_onestep()[0][0]])
        f.close()
        out["out_optional"] = {"text": p.read_text(), "columns": cols, "rows": rows}
        p = Path(d) / "run.dcd"
        with open(p, "wb") as fh:
            sdcd.write_header(fh, 5, True)
            for x in DCD_FRAMES:
                sdcd.write_frame(fh, np.array(x), DCD_BOX, fix_com_origin=True)
        f = rdcd.DcdFile(str(p))
        f.open_to_read()
        f.read_header()
        h = f.get_header()
        frames = []
        while f.has_more_data():
            frames.append(f.read_onestep())
        f.close()
        out["dcd"] = {"bytes_hex": p.read_bytes().hex(), "with_unit_cell": bool(h.with_unit_cell),
                      "nmp_real": int(h.nmp_real), "frames": frames}
    out["frames"] = FRAMES
    out["bp_frames"] = BP_FRAMES
    out["opt_frames"] = OPT_FRAMES
    out["dcd_frames"] = DCD_FRAMES
    out["dcd_box"] = DCD_BOX
    (Path(__file__).parent / "outputs.json").write_text(json.dumps(out, indent=1))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_output_fixtures.py <path of the SIS source tree>")
    main(Path(sys.argv[1]))
