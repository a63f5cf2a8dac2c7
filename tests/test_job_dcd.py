"""Trajectory re-analysis (job_dcd.F90:64-79) on the GPU: the 25 frames of
the reference's CAG47 regression trajectory (check/test_DCD_CAG47) as 25
instances of one context, against the reference's golden energies (same
bars as the oracle's own golden test) and against the oracle frame by frame.
A DCD round trip through the package's writer and reader feeds the same
frames back."""
import numpy as np
import pytest

from helpers import GOLDEN, cag47_system
from oracle.oracle import Oracle
from sis_gb300 import FP64, MIXED
from sis_gb300.dcd import write_dcd
from sis_gb300.job_dcd import dcd_energies, frame_energies

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cag47():
    z = np.load(GOLDEN / "cag47.npz")
    s = cag47_system(0)
    inst = s.instances[0]
    return s, inst, z["xyz"].astype(np.float64), z["energy"]


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_cag47_frames_match_golden_energies(prec, cag47):
    s, inst, frames, golden = cag47
    E = frame_energies(s.ff, s.opts, inst.chains, frames, inst.tempK, inst.ionic_strength, precision=prec)
    # golden columns: step, Ebond, Eangl, Eexv, Eele, -, Ebp, -; frames are stored in FP32
    assert np.all(np.abs(E[:, 1] - golden[:, 1]) <= 1e-4 * np.abs(golden[:, 1]) + 1e-4)
    assert np.all(np.abs(E[:, 2] - golden[:, 2]) <= 1e-4 * np.abs(golden[:, 2]) + 1e-4)
    assert np.all(np.abs(E[:, 5] - golden[:, 3]) <= 2e-3 * np.abs(golden[:, 3]) + 1e-5)
    assert np.all(np.abs(E[:, 6] - golden[:, 4]) <= 6e-3 * np.abs(golden[:, 4]))


def test_cag47_frames_match_oracle(cag47, tmp_path):
    s, inst, frames, golden = cag47
    path = tmp_path / "cag47.dcd"
    write_dcd(path, list(frames))
    E = dcd_energies(path, s.ff, s.opts, inst.chains, inst.tempK, inst.ionic_strength, precision=FP64)
    orc = Oracle.from_instance(s, 0)
    for f in range(len(frames)):
        orc.set_xyz(0, frames[f].astype(np.float32).astype(np.float64))
        orc.neighbor_list(0)
        orc.set_bp_energy_flag(0)
        ref = orc.energy_sumup(0)
        scale = np.abs(ref[1:7]).sum()
        for k in range(1, 7):
            assert abs(E[f, k] - ref[k]) <= 1e-12 * max(abs(ref[k]), 1e-3 * scale), (f, k)
