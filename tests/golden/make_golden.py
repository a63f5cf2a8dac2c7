"""Builds the golden fixtures of tests/golden/ from the reference tree.

Run where the reference is present (it is read-only and absent on GPU hosts;
the fixtures are committed):

    python tests/golden/make_golden.py <path of the SIS source tree>

Fixtures written:

* ``cag47.npz`` -- every 4th frame of ``check/test_DCD_CAG47/CAG47.dcd``
  (141 beads, written by OpenMM) with the matching rows of
  ``CAG47.energy.out`` (step, Ebond, Eangl, Eexv, Eele, -, Ebp, -) and the
  sequence of ``CAG47.fasta``.  The reference's own regression test
  (``check/test_DCD_CAG47/run_test_DCD_CAG47.sh``) compares SIS against these
  energies at 295.15 K, 0.15 M, DH cutoff 50 A, length_per_charge 4.38178046,
  with bond k=15 r0=5.9, angle k=10 a0=2.618, WCA sigma=10 eps=2
  (``para/rna_NHT22.ff``), no dihedral term.
* ``test_md.npz`` -- the first and last frame of ``check/test_md.dcd``
  (564 beads = four CAG47 chains in a PBC box given by its unit-cell record).
* ``t2s2hp.npz`` -- ``check/T2S2HP.fasta`` and ``check/T2S2HP_random.xyz``
  (27 nt), the input of ``check/input_T2S2HP.toml`` (model 5, ReB angle,
  exponential dihedral, DH cutoff type 2).
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from sis_gb300.dcd import read_dcd  # noqa: E402
from sis_gb300.inputs import read_fasta, read_xyz  # noqa: E402


def main(ref: Path):
    d = ref / "check" / "test_DCD_CAG47"
    frames, _ = read_dcd(d / "CAG47.dcd")
    ene = np.loadtxt(d / "CAG47.energy.out")
    seq = "".join("AUGCD"[s] for s in read_fasta(d / "CAG47.fasta")[0].seq)
    sel = np.arange(0, len(frames), 4)
    np.savez_compressed(HERE / "cag47.npz", xyz=frames[sel].astype(np.float32), energy=ene[sel], seq=np.array(seq))
    frames, boxes = read_dcd(ref / "check" / "test_md.dcd")
    np.savez_compressed(HERE / "test_md.npz", xyz=frames[[0, -1]].astype(np.float32), box=boxes[[0, -1]])
    c = ref / "check"
    seq2 = "".join("AUGCD"[s] for s in read_fasta(c / "T2S2HP.fasta")[0].seq)
    np.savez_compressed(HERE / "t2s2hp.npz", xyz=read_xyz(c / "T2S2HP_random.xyz"), seq=np.array(seq2))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the SIS source tree>")
    main(Path(sys.argv[1]))
