"""Regenerates the force-field parameter files of this directory from the
reference's own .ff files (Hori-Lab/SIS ``sis.ff`` and
``check/sis_dih_ReB_NN.ff``), re-serialised as plain TOML with the same keys
so that the engine's .ff reader (sis_gb300/inputs.py) reads them as it reads
the originals.  Run only where the reference tree is present:

    python sis_gb300/data/make_ff.py <path of the SIS source tree>
"""
import sys
import tomllib
from pathlib import Path

HERE = Path(__file__).resolve().parent
FILES = {"sis.ff": "sis.ff", "check/sis_dih_ReB_NN.ff": "sis_dih_ReB_NN.ff"}


def dump(d, prefix=""):
    lines, subs = [], []
    for k, v in d.items():
        if isinstance(v, dict):
            subs.append((k, v))
        elif isinstance(v, bool):
            lines.append(f"{k} = {'true' if v else 'false'}")
        elif isinstance(v, str):
            lines.append(f'{k} = "{v}"')
        else:
            lines.append(f"{k} = {v!r}")
    out = []
    if lines:
        if prefix:
            out.append(f"[{prefix}]")
        out += lines
        out.append("")
    for k, v in subs:
        out += dump(v, f"{prefix}.{k}" if prefix else k)
    return out


def main(ref):
    for src, dst in FILES.items():
        t = tomllib.loads((Path(ref) / src).read_text())
        (HERE / dst).write_text("\n".join(dump(t)))
        print("wrote", HERE / dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python sis_gb300/data/make_ff.py <path of the SIS source tree>")
    main(sys.argv[1])
