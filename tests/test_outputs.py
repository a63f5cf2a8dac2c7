"""Output files in the reference's formats (sis_gb300.outputs).

CPU: Fortran G/E/F editing, the .out (with and without optional columns),
.bp and .dcd files against tests/golden/outputs.json (written by
tests/golden/make_output_fixtures.py, which parsed them with the
reference's own readers, utils/sisout.py, utils/sisbp.py and utils/dcd.py),
.bpe lines and the .rst block layout.
GPU: a run restarted from its .rst file continues bit for bit, and the
per-frame writers write what the engine holds.
"""
import json
import struct
from pathlib import Path

import numpy as np
import pytest

from sis_gb300.outputs import (BOLTZ_KCAL_MOL, RST_PBC, RST_REPLICA, RST_STEP, RST_XYZ, BpeFile, BpFile, OutFile,
                               formed_pairs, fortran_g, read_bp, read_out, read_rst, restart_engine, save_frame,
                               write_rst)

GOLDEN = json.loads((Path(__file__).parent / "golden" / "outputs.json").read_text())


@pytest.mark.parametrize("x,expect", [
    (1.0, "  1.00000    "),
    (0.0, "  0.00000    "),
    (0.1, " 0.100000    "),
    (-0.05, "-0.500000E-01"),
    (123.4567, "  123.457    "),
    (999999.4, "  999999.    "),
    (999999.6, " 0.100000E+07"),
    (-1.0e-7, "-0.100000E-06"),
    (1.0e100, " 0.100000+101"),
    (-12345.67, " -12345.7    "),
])
def test_fortran_g_editing(x, expect):
    """G13.6: F(w-4).(d-k) and four blanks when the value rounded to six
    digits lies in [0.1, 10**6), otherwise E13.6; zero as F9.5."""
    assert fortran_g(x) == expect
    assert len(fortran_g(x)) == 13


@pytest.mark.parametrize("replica", [False, True])
def test_out_file_matches_the_reference_reader(replica, tmp_path):
    g = GOLDEN[f"out_replica{int(replica)}"]
    p = tmp_path / "a.out"
    w = OutFile(p, replica=replica, ele=True)
    for k, (step, T, ekin, e) in enumerate(GOLDEN["frames"]):
        w.write(step, T, ekin, e, rep_label=k + 1 if replica else None)
    w.close()
    assert p.read_text() == g["text"]
    cols = read_out(p)
    assert list(cols) == (["nframe", "R", "T"] if replica else ["nframe", "T"]) + [
        "Ekin", "Epot", "Ebond", "Eangl", "Edih", "Ebp", "Eexv", "Eele"]
    got = np.array(list(cols.values())).T
    assert np.array_equal(got, np.array(g["rows"]))
    # columns as the reference's reader maps them
    names = {"step": "nframe", "label": "R", "temp": "T", "e_kin": "Ekin", "e_pot": "Epot", "e_bond": "Ebond",
             "e_angl": "Eangl", "e_dih": "Edih", "e_bp": "Ebp", "e_exv": "Eexv", "e_ele": "Eele"}
    assert {names[k]: v for k, v in g["columns"].items()} == {n: i for i, n in enumerate(cols)}
    # six significant digits of every energy
    for (step, T, ekin, e), row in zip(GOLDEN["frames"], g["rows"]):
        vals = [ekin] + list(e[:6]) + [e[6]]
        assert np.allclose(row[-8:], vals, rtol=5e-6, atol=0)


def test_bp_file_matches_the_reference_reader(tmp_path):
    p = tmp_path / "a.bp"
    w = BpFile(p)
    for pairs, st, ene in GOLDEN["bp_frames"]:
        w.write_frame(np.array(pairs), np.array(st), np.array(ene), 300.0)
    w.close()
    assert p.read_bytes().hex() == GOLDEN["bp"]["bytes_hex"]
    frames = read_bp(p)
    ref = GOLDEN["bp"]["frames"]
    assert [[(i, j) for i, j, _ in f] for f in frames] == [[tuple(q) for q in f["pairs"]] for f in ref]
    assert [[e for _, _, e in f] for f in frames] == [f["energies"] for f in ref]


def test_out_optional_columns_match_the_reference_reader(tmp_path):
    """Estage and Etweezers after Eele (write_out.F90); the reference's
    reader files the Etweezers column under e_stage, and that is what the
    fixture records."""
    g = GOLDEN["out_optional"]
    p = tmp_path / "a.out"
    w = OutFile(p, ele=True, stage=True, twz=True)
    for step, T, ekin, e, rg in GOLDEN["opt_frames"]:
        w.write(step, T, ekin, e, rg=rg)
    w.close()
    assert p.read_text() == g["text"]
    cols = read_out(p)
    assert list(cols)[-3:] == ["Eele", "Estage", "Etweezers"]
    assert np.array_equal(np.array(list(cols.values())).T, np.array(g["rows"]))
    assert g["columns"]["e_ele"] == 9 and g["columns"]["e_stage"] == 11


def test_dcd_matches_the_reference_reader(tmp_path):
    """Unit-cell records and centroid-relative coordinates
    (fix_com_origin), read back by the reference's utils/dcd.py."""
    from sis_gb300 import dcd
    g = GOLDEN["dcd"]
    p = tmp_path / "a.dcd"
    with open(p, "wb") as f:
        dcd.write_header(f, 5, True)
        for x in GOLDEN["dcd_frames"]:
            dcd.write_frame(f, np.array(x), GOLDEN["dcd_box"], fix_com_origin=True)
    assert p.read_bytes().hex() == g["bytes_hex"]
    assert g["with_unit_cell"] and g["nmp_real"] == 5
    frames, boxes = dcd.read_dcd(p)
    assert np.array_equal(frames, np.array(g["frames"]))
    assert np.array_equal(boxes, [GOLDEN["dcd_box"]] * 2)
    for x, fr in zip(GOLDEN["dcd_frames"], frames):
        x = np.array(x)
        assert np.allclose(fr, x - x.mean(axis=0), rtol=0, atol=1e-6)


def test_bpall_and_bpe(tmp_path):
    pairs, st, ene = GOLDEN["bp_frames"][0]
    kT = 300.0 * BOLTZ_KCAL_MOL
    assert formed_pairs(np.array(pairs), st, ene, 300.0) == [(5, 20, -3.2), (30, 44, -1.5)]
    assert -0.4 > -kT  # the (6, 19) pair is formed but above -kT
    p = tmp_path / "a.bpall"
    w = BpFile(p, all_formed=True)
    w.write_frame(np.array(pairs), np.array(st), np.array(ene), 300.0)
    w.close()
    assert [(i, j) for i, j, _ in read_bp(p)[0]] == [(5, 20), (6, 19), (30, 44)]
    p = tmp_path / "a.bpe"
    w = BpeFile(p)
    w.write_frame(np.array(pairs), np.array(st), np.array(ene), 300.0)
    w.write_frame(np.zeros((0, 7), dtype=int), [], [], 300.0)
    w.close()
    assert p.read_text() == "     5    20  -3.20    30    44  -1.50\n\n"


def test_rst_blocks(tmp_path):
    rng = np.random.default_rng(1)
    x, v, a = rng.normal(size=(3, 7, 3))
    p = tmp_path / "a.rst"
    write_rst(p, 123456789012, x, v, a, grep=2, box=[100.0, 110.0, 120.0], rep2lab=[3, 1, 2])
    b = p.read_bytes()
    # replica table first (write_rst.F90:45-54), then the step block
    assert struct.unpack("<iii", b[:12]) == (RST_REPLICA, 4 * 7, 3)
    off = 8 + 4 * 7
    assert struct.unpack("<iiiq", b[off:off + 20]) == (RST_STEP, 12, 1, 123456789012)
    off += 20
    assert struct.unpack("<iiii", b[off:off + 16]) == (RST_XYZ, 8 + 8 * 21, 2, 7)
    assert struct.unpack("<ii", b[-32:-24]) == (RST_PBC, 24)
    r = read_rst(p)
    assert r.step == 123456789012 and r.rep2lab == [3, 1, 2]
    assert np.array_equal(r.xyz[2], x) and np.array_equal(r.velos[2], v) and np.array_equal(r.accels[2], a)
    assert np.array_equal(r.box, [100.0, 110.0, 120.0])


def _hairpin(ff):
    from sis_gb300.coil import random_coil
    from sis_gb300.model import Chain, Instance, Options, System

    rng = np.random.default_rng(5)
    x = random_coil(rng, 30, amin_deg=60.0, amax_deg=100.0, rmin=3.0)
    inst = Instance([Chain.from_string("GGGGCAAAAGCCCCAAAAGGGGAAAACCCC")], tempK=300.0, ionic_strength=0.15, xyz=x)
    return System(ff, Options(bp_model=1), [inst])


@pytest.mark.gpu
def test_restart_file_continues_bit_for_bit(sis_ff, tmp_path):
    """A run saved to .rst at step 40 and a fresh context loaded from it take
    the same next 60 steps bit for bit: the Philox noise is keyed by the
    step the file stores.  The first run reloads its own state at the same
    point, since a loaded state rebuilds the lists (as the reference
    rebuilds them on a restart), and list order enters the FP32 sums."""
    from sis_gb300 import MIXED
    from sis_gb300.engine import Engine

    sysm = _hairpin(sis_ff)
    a = Engine(sysm, precision=MIXED, seed=8)
    a.set_force_cap(1000.0)
    a.init_velocities()
    a.step(40)
    x, v, acc = a.get_state(0)
    write_rst(tmp_path / "a.rst", a.get_step(), x, v, acc)
    a.set_state(0, x, v, acc)
    a.step(60)
    b = Engine(sysm, precision=MIXED, seed=8)
    b.set_force_cap(1000.0)
    r = restart_engine(b, tmp_path / "a.rst")
    assert r.step == 40 and b.get_step() == 40
    b.step(60)
    for u, w in zip(a.get_state(0), b.get_state(0)):
        assert np.array_equal(u, w)


@pytest.mark.gpu
def test_frame_writers_write_what_the_engine_holds(sis_ff, tmp_path):
    from sis_gb300 import FP64
    from sis_gb300.engine import Engine

    sysm = _hairpin(sis_ff)
    eng = Engine(sysm, precision=FP64, seed=3)
    eng.set_force_cap(1000.0)
    eng.init_velocities()
    out, bp, bpe = OutFile(tmp_path / "a.out"), BpFile(tmp_path / "a.bp"), BpeFile(tmp_path / "a.bpe")
    want_pairs, want_e = [], []
    for k in range(3):
        eng.step(50)
        save_frame(eng, 0, eng.get_step(), out=out, bp=bp, bpe=bpe)
        want_pairs.append(formed_pairs(eng.get_list(0, 2), eng.get_bp_status(0), eng.get_bp_energies(0), 300.0))
        want_e.append([eng.energy_kinetic(0)] + list(eng.energy_sumup(0)[:7]))
    for w in (out, bp, bpe):
        w.close()
    cols = read_out(tmp_path / "a.out")
    assert list(cols["nframe"]) == [50, 100, 150]
    got = np.array([cols[n] for n in ("Ekin", "Epot", "Ebond", "Eangl", "Edih", "Ebp", "Eexv", "Eele")]).T
    assert np.allclose(got, np.array(want_e), rtol=5e-6, atol=1e-6)
    frames = read_bp(tmp_path / "a.bp")
    assert [[(i, j) for i, j, _ in f] for f in frames] == [[(i, j) for i, j, _ in p] for p in want_pairs]
    assert all(np.allclose([e for *_, e in f], [e for *_, e in p], rtol=1e-6) for f, p in zip(frames, want_pairs))
    assert len((tmp_path / "a.bpe").read_text().splitlines()) == 3


class _KeyedEngine:
    """What restart_engine needs of an engine, with a noise key."""

    def __init__(self, seed, stream, n=7):
        self.seed, self.streams, self.n = seed, [stream], n
        self.loaded = None

    def nmp(self, inst):
        return self.n

    def set_state(self, inst, x, v, a):
        self.loaded = (x, v, a)

    def set_step(self, s):
        self.step = s


def test_rst_noise_key(tmp_path):
    """The engine's Philox key and stream go into a block the reference's
    reader skips by size; a restart into an engine with another key is
    refused unless asked for, since the run would draw other noise."""
    from sis_gb300.outputs import RST_NOISE
    x = np.zeros((7, 3))
    p = tmp_path / "a.rst"
    write_rst(p, 10, x, x, x, grep=2, noise=(2 ** 63 + 5, 7))
    b = p.read_bytes()
    assert struct.unpack("<iiiIQ", b[-24:]) == (RST_NOISE, 16, 2, 7, 2 ** 63 + 5)
    assert read_rst(p).noise == {2: (2 ** 63 + 5, 7)}
    eng = _KeyedEngine(2 ** 63 + 5, 7)
    restart_engine(eng, p, grep=2)
    assert eng.step == 10 and eng.loaded is not None
    with pytest.raises(ValueError, match="noise key"):
        restart_engine(_KeyedEngine(2 ** 63 + 5, 8), p, grep=2)
    with pytest.raises(ValueError, match="noise key"):
        restart_engine(_KeyedEngine(12345, 7), p, grep=2)
    restart_engine(_KeyedEngine(12345, 7), p, grep=2, check_noise=False)


@pytest.mark.parametrize("cut", [10, 100, -5, -40])
def test_truncated_dcd_raises(tmp_path, cut):
    from sis_gb300 import dcd
    p = tmp_path / "a.dcd"
    dcd.write_dcd(p, [np.zeros((4, 3)), np.ones((4, 3))], box=(10.0, 10.0, 10.0))
    b = p.read_bytes()
    frames, _ = dcd.read_dcd(p)
    assert frames.shape == (2, 4, 3)
    p.write_bytes(b[:cut])
    with pytest.raises(ValueError, match="truncated DCD"):
        dcd.read_dcd(p)


@pytest.mark.parametrize("cut,what", [(5, "header"), (-3, "record"), (-8, "terminator")])
def test_truncated_bp_raises(tmp_path, cut, what):
    p = tmp_path / "a.bp"
    w = BpFile(p)
    for pairs, st, ene in GOLDEN["bp_frames"]:
        w.write_frame(np.array(pairs), np.array(st), np.array(ene), 300.0)
    w.close()
    assert len(read_bp(p)) == 2
    p.write_bytes(p.read_bytes()[:cut])
    with pytest.raises(ValueError, match=what):
        read_bp(p)
