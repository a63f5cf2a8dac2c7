"""ctypes wrapper of the CPU FP64 oracle (oracle/_build/libsis_oracle.so).

TEST INFRASTRUCTURE ONLY: the correctness oracle and the timed CPU baseline.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm may import this module.  The product (sis_gb300, libsisgpu.so) never
imports, links or calls it.

One :class:`Oracle` holds one reference "job": a topology with nrep replicas
of it (the reference's xyz(3,nmp,nrep_proc)).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path
from typing import Sequence

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libsis_oracle.so"


class or_params(C.Structure):
    _fields_ = [
        ("bond_k", C.c_double), ("bond_r0", C.c_double),
        ("angl_reb", C.c_int32), ("angl_k", C.c_double), ("angl_t0", C.c_double),
        ("dih_type", C.c_int32), ("dih_k", C.c_double), ("dih_w", C.c_double), ("dih_p0", C.c_double),
        ("wca_sigma", C.c_double), ("wca_eps", C.c_double),
        ("bp_model", C.c_int32), ("bp_min_loop", C.c_int32), ("bp_jnext_compat", C.c_int32),
        ("bp_cutoff_energy", C.c_double),
        ("bp_ff", (C.c_double * 15) * 3),
        ("nn_dH", C.c_double * 21), ("nn_dS", C.c_double * 21), ("dH0", C.c_double), ("dS0", C.c_double),
        ("nnend", C.c_int32), ("nnend_dH", C.c_double * 6), ("nnend_dS", C.c_double * 6),
        ("dHend0", C.c_double), ("dSend0", C.c_double),
        ("flg_ele", C.c_int32), ("ele_cutoff_type", C.c_int32),
        ("ele_cutoff_inp", C.c_double), ("length_per_charge", C.c_double),
        ("ele_excl_bond", C.c_int32), ("ele_excl_angle", C.c_int32),
        ("temp_independent", C.c_int32), ("tempK_ref", C.c_double),
        ("integrator", C.c_int32), ("dt", C.c_double), ("viscosity_Pas", C.c_double), ("nl_margin", C.c_double),
        ("nstep_bp_mc", C.c_int32), ("max_bp_per_nt", C.c_int32),
    ]


_lib = None


def build(force: bool = False) -> Path:
    """Builds the oracle with the recipe of oracle/Makefile (g++ directly when
    make is absent)."""
    import shutil

    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < max(
            p.stat().st_mtime for p in [HERE / "sis_oracle.cpp", HERE / "sis_oracle.h"]):
        if shutil.which("make"):
            subprocess.run(["make", "-s", "-C", str(HERE), "-B" if force else "all"], check=True)
        else:
            LIB_PATH.parent.mkdir(exist_ok=True)
            subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared", "-o",
                            str(LIB_PATH), str(HERE / "sis_oracle.cpp")], check=True)
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB_PATH))
        vp, i32, d, i64 = C.c_void_p, C.c_int32, C.c_double, C.c_int64
        sig = {
            "or_create": (vp, [i32, vp, vp, vp, vp, i32, vp, vp, vp, C.POINTER(or_params)]),
            "or_destroy": (None, [vp]),
            "or_nmp": (i32, [vp]),
            "or_set_xyz": (None, [vp, i32, vp]), "or_get_xyz": (None, [vp, i32, vp]),
            "or_set_velos": (None, [vp, i32, vp]), "or_get_velos": (None, [vp, i32, vp]),
            "or_set_accels": (None, [vp, i32, vp]), "or_get_accels": (None, [vp, i32, vp]),
            "or_neighbor_list": (None, [vp, i32]),
            "or_get_list": (i32, [vp, i32, i32, vp, i32]),
            "or_get_bp_coef": (i32, [vp, i32, vp, i32]),
            "or_force": (None, [vp, i32, vp]),
            "or_force_mc": (None, [vp, i32, vp]),
            "or_get_mc_draws": (i32, [vp, vp, i32]),
            "or_get_bp_status": (i32, [vp, i32, vp, i32]),
            "or_force_term": (None, [vp, i32, i32, vp]),
            "or_energy_sumup": (None, [vp, i32, d, vp]),
            "or_energy_kinetic": (d, [vp, i32]),
            "or_rg": (d, [vp, i32]),
            "or_set_bp_energy_flag": (None, [vp, i32]),
            "or_get_bp_state": (i32, [vp, i32, vp, vp, i32]),
            "or_get_ele": (None, [vp, i32, vp]),
            "or_get_md_coef": (None, [vp, i32, vp]),
            "or_get_bp_paras": (None, [vp, vp, vp]),
            "or_get_bp3_tables": (None, [vp, vp, vp]),
            "or_set_temperature": (None, [vp, i32, d, d]),
            "or_run": (i64, [vp, i64, vp]),
            "or_md_init": (None, [vp]),
            "or_init_velocities": (None, [vp]),
            "or_nrebuild": (i64, [vp]),
            "or_mt_create": (vp, [i32]), "or_mt_destroy": (None, [vp]),
            "or_mt_int32": (C.c_uint32, [vp]), "or_mt_double1": (d, [vp]), "or_mt_double3": (d, [vp]),
            "or_mt_boxmuller": (d, [vp]),
            "or_seed": (None, [vp, i32]),
            "or_mt_jump": (None, [vp, i32, i32, vp]),
            "or_seed_streams": (None, [vp, i32, i32]),
            "or_const": (d, [i32]),
            "or_set_stage": (None, [vp, d, d]),
            "or_set_rg_bias": (None, [vp, i32, d, vp]),
            "or_set_restraints": (None, [vp, i32, vp, vp]),
            "or_set_tweezers": (None, [vp, i32, vp, vp, i32, vp, vp, vp, vp]),
            "or_set_frozen": (None, [vp, i32, vp]),
            "or_set_ss_pairs": (None, [vp, i32, vp]),
            "or_set_bias_ss": (None, [vp, i32, d]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype, fn.argtypes = res, args
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def pack(ff, o) -> or_params:
    p = or_params()
    p.bond_k, p.bond_r0 = ff.bond_k, ff.bond_r0
    p.angl_reb, p.angl_k, p.angl_t0 = int(ff.angl_reb), ff.angl_k, ff.angl_t0
    p.dih_type, p.dih_k, p.dih_w, p.dih_p0 = ff.dih_type, ff.dih_k, ff.dih_w, ff.dih_p0
    p.wca_sigma, p.wca_eps = ff.wca_sigma, ff.wca_eps
    p.bp_model, p.bp_min_loop, p.bp_jnext_compat = o.bp_model, o.bp_min_loop, int(o.bp_jnext_compat)
    p.bp_cutoff_energy = ff.bp_cutoff_energy
    bpa = ff.bp_array()
    for t in range(3):
        for k in range(15):
            p.bp_ff[t][k] = bpa[t, k]
    for k in range(21):
        p.nn_dH[k], p.nn_dS[k] = ff.nn_dH[k], ff.nn_dS[k]
    p.dH0, p.dS0, p.nnend = ff.dH0, ff.dS0, int(ff.nnend)
    for k in range(6):
        p.nnend_dH[k], p.nnend_dS[k] = ff.nnend_dH[k], ff.nnend_dS[k]
    p.dHend0, p.dSend0 = ff.dHend0, ff.dSend0
    p.flg_ele, p.ele_cutoff_type = int(o.flg_ele), o.ele_cutoff_type
    p.ele_cutoff_inp, p.length_per_charge = o.ele_cutoff, o.length_per_charge
    p.ele_excl_bond, p.ele_excl_angle = int(o.ele_excl_bond), int(o.ele_excl_angle)
    p.temp_independent, p.tempK_ref = o.temp_independent, o.tempK_ref
    p.integrator, p.dt, p.viscosity_Pas, p.nl_margin = o.integrator, o.dt, o.viscosity_Pas, o.nl_margin
    p.nstep_bp_mc, p.max_bp_per_nt = o.nstep_bp_mc, o.max_bp_per_nt
    return p


class Oracle:
    """The reference's module state for one topology and nrep replicas."""

    def __init__(self, ff, opts, chains, tempK: Sequence[float], ionic: Sequence[float], box=None, has_charge=None):
        self.L = lib()
        self.nrep = len(tempK)
        self._lens = np.asarray([len(c) for c in chains], dtype=np.int32)
        self._types = np.asarray([c.moltype for c in chains], dtype=np.int32)
        self._seq = np.ascontiguousarray(np.concatenate([c.seq for c in chains]), dtype=np.int32)
        if has_charge is None:
            has_charge = (self._seq != 4).astype(np.uint8)
        self._chg = np.ascontiguousarray(has_charge, dtype=np.uint8)
        self._T = np.asarray(tempK, dtype=np.float64)
        self._I = np.asarray(ionic, dtype=np.float64)
        self._box = None if box is None else np.asarray(box, dtype=np.float64)
        self._par = pack(ff, opts)
        self.h = self.L.or_create(len(chains), _p(self._lens), _p(self._types), _p(self._seq), _p(self._chg), self.nrep,
                                  _p(self._T), _p(self._I), _p(self._box), C.byref(self._par))
        self.nmp = int(self.L.or_nmp(self.h))

    @classmethod
    def from_instance(cls, system, k: int):
        inst = system.instances[k]
        o = cls(system.ff, system.opts, inst.chains, [inst.tempK], [inst.ionic_strength], inst.box, inst.charges())
        if inst.xyz is not None:
            o.set_xyz(0, inst.xyz)
        return o

    def __del__(self):
        try:
            self.L.or_destroy(self.h)
        except Exception:
            pass

    def set_xyz(self, r, x):
        self.L.or_set_xyz(self.h, r, _p(np.ascontiguousarray(x, dtype=np.float64)))

    def get_xyz(self, r=0):
        x = np.empty((self.nmp, 3))
        self.L.or_get_xyz(self.h, r, _p(x))
        return x

    def set_velos(self, r, v):
        self.L.or_set_velos(self.h, r, _p(np.ascontiguousarray(v, dtype=np.float64)))

    def get_velos(self, r=0):
        x = np.empty((self.nmp, 3))
        self.L.or_get_velos(self.h, r, _p(x))
        return x

    def set_accels(self, r, a):
        self.L.or_set_accels(self.h, r, _p(np.ascontiguousarray(a, dtype=np.float64)))

    def get_accels(self, r=0):
        x = np.empty((self.nmp, 3))
        self.L.or_get_accels(self.h, r, _p(x))
        return x

    def neighbor_list(self, r=0):
        self.L.or_neighbor_list(self.h, r)

    def get_list(self, r, kind):
        w = 7 if kind == 2 else 2
        n = self.L.or_get_list(self.h, r, kind, None, 0)
        out = np.zeros((max(n, 1), w), dtype=np.int32)
        self.L.or_get_list(self.h, r, kind, _p(out), n)
        return out[:n]

    def get_bp_coef(self, r=0):
        n = self.L.or_get_bp_coef(self.h, r, None, 0)
        out = np.zeros((max(n, 1), 2))
        self.L.or_get_bp_coef(self.h, r, _p(out), n)
        return out[:n]

    def force(self, r=0):
        f = np.empty((self.nmp, 3))
        self.L.or_force(self.h, r, _p(f))
        return f

    def force_mc(self, r=0):
        """Forces with the base-pair Monte Carlo removal (force_bp_limit_triplet)."""
        f = np.zeros((self.nmp, 3))
        self.L.or_force_mc(self.h, r, _p(f))
        return f

    def mc_draws(self):
        n = self.L.or_get_mc_draws(self.h, None, 0)
        out = np.zeros(n)
        self.L.or_get_mc_draws(self.h, _p(out), n)
        return out

    def bp_state(self, r=0):
        """(energy, status) of every base-pair record of the last force evaluation."""
        n = self.L.or_get_bp_state(self.h, r, None, None, 0)
        e = np.zeros(n)
        st = np.zeros(n, dtype=np.uint8)
        self.L.or_get_bp_state(self.h, r, _p(e), st.ctypes.data_as(C.c_void_p), n)
        return e, st

    def bp_status(self, r=0):
        n = self.L.or_get_bp_status(self.h, r, None, 0)
        out = np.zeros(n, dtype=np.uint8)
        self.L.or_get_bp_status(self.h, r, out.ctypes.data_as(C.c_void_p), n)
        return out

    # optional terms (force.F90:62-75): force term 7, energy slots 7-10
    def set_stage(self, sigma, eps):
        self.L.or_set_stage(self.h, float(sigma), float(eps))

    def set_rg_bias(self, k, rg0, flat=False, off=False):
        r0 = np.broadcast_to(np.asarray(rg0, dtype=np.float64), (self.nrep,)).copy()
        self._rg0 = r0
        self.L.or_set_rg_bias(self.h, 0 if off else (2 if flat else 1), float(k), _p(r0))

    def set_restraints(self, restraints):
        ids = np.array([[q.i, q.j, 2 if q.to_bead else 1] for q in restraints], dtype=np.int32).reshape(-1, 3)
        par = np.array([[q.eps, q.d, q.s, q.rcut] for q in restraints], dtype=np.float64).reshape(-1, 4)
        self._rest = (ids, par)
        self.L.or_set_restraints(self.h, len(restraints), _p(ids), _p(par))

    def set_tweezers(self, dcf=(), fr=()):
        """dcf: ConstantForcePair (same force in every replica); fr: ForceRampPair."""
        dp = np.array([[q.i, q.j] for q in dcf], dtype=np.int32).reshape(-1, 2)
        df = np.ascontiguousarray(np.broadcast_to(np.array([q.force for q in dcf], dtype=np.float64).reshape(-1, 3),
                                                  (self.nrep, len(dcf), 3)))
        fp = np.array([[q.i, q.j] for q in fr], dtype=np.int32).reshape(-1, 2)
        fk = np.array([q.k for q in fr], dtype=np.float64).reshape(-1, 2)
        fi = np.array([q.init for q in fr], dtype=np.float64).reshape(-1, 2, 3)
        fv = np.array([q.velo for q in fr], dtype=np.float64).reshape(-1, 2, 3)
        self._twz = (dp, df, fp, fk, fi, fv)
        self.L.or_set_tweezers(self.h, len(dcf), _p(dp), _p(df), len(fr), _p(fp), _p(fk), _p(fi), _p(fv))

    def set_ss_pairs(self, pairs):
        """read_ss.F90 bp_map: base pairs only between these (imp, jmp), 1-based."""
        a = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
        self._ss = a
        self.L.or_set_ss_pairs(self.h, a.shape[0], _p(a))

    def set_bias_ss(self, force_kcal_per_mol_A, on=True):
        """[Bias_SS]: constant pull of allowed pairs outside the distance window."""
        self.L.or_set_bias_ss(self.h, int(on), float(force_kcal_per_mol_A))

    def set_frozen(self, beads):
        """[Freeze]: 1-based bead numbers whose positions stay fixed."""
        b = np.ascontiguousarray(beads, dtype=np.int32)
        self._frozen = b
        self.L.or_set_frozen(self.h, b.size, _p(b))

    def force_term(self, r, term):
        f = np.empty((self.nmp, 3))
        self.L.or_force_term(self.h, r, term, _p(f))
        return f

    def energy_sumup(self, r=0, tempK=None):
        e = np.zeros(11)
        T = self._T[r] if tempK is None else tempK
        self.L.or_energy_sumup(self.h, r, float(T), _p(e))
        return e

    def energy_kinetic(self, r=0):
        return float(self.L.or_energy_kinetic(self.h, r))

    def rg(self, r=0):
        return float(self.L.or_rg(self.h, r))

    def set_bp_energy_flag(self, f):
        self.L.or_set_bp_energy_flag(self.h, int(f))

    def get_ele(self, r=0):
        o = np.zeros(4)
        self.L.or_get_ele(self.h, r, _p(o))
        return o

    def get_md_coef(self, r=0):
        o = np.zeros((self.nmp, 4))
        self.L.or_get_md_coef(self.h, r, _p(o))
        return o

    def get_bp_paras(self):
        o = np.zeros((6, 16))
        c = np.zeros(1)
        self.L.or_get_bp_paras(self.h, _p(o), _p(c))
        return o, float(c[0])

    def get_bp3_tables(self):
        a, b = np.zeros(468), np.zeros(468)
        self.L.or_get_bp3_tables(self.h, _p(a), _p(b))
        return a, b

    def md_init(self):
        self.L.or_md_init(self.h)

    def init_velocities(self):
        self.L.or_init_velocities(self.h)

    def seed_streams(self, seed, replica_run=False):
        """Replica noise streams as the reference derives them (init_mts.F90):
        stream (replica + 1 + replica_run) * 2^256 outputs ahead of the
        MT19937 stream initialised by `seed`."""
        self.L.or_seed_streams(self.h, int(seed), int(bool(replica_run)))

    def seed(self, s):
        self.L.or_seed(self.h, int(s))

    def run(self, nsteps, noise=None):
        if noise is not None:
            noise = np.ascontiguousarray(noise, dtype=np.float64)
        return int(self.L.or_run(self.h, int(nsteps), _p(noise)))

    def nrebuild(self):
        return int(self.L.or_nrebuild(self.h))


class MT:
    """MT19937 stream with the reference's double draws and polar Box-Muller."""

    def __init__(self, seed: int):
        self.L = lib()
        self.h = self.L.or_mt_create(int(seed))

    def __del__(self):
        try:
            self.L.or_mt_destroy(self.h)
        except Exception:
            pass

    def int32(self):
        return int(self.L.or_mt_int32(self.h))

    def double1(self):
        return float(self.L.or_mt_double1(self.h))

    def double3(self):
        return float(self.L.or_mt_double3(self.h))

    def boxmuller(self):
        return float(self.L.or_mt_boxmuller(self.h))

    def jumped(self, jp: int, stream_id: int) -> "MT":
        """A new stream stream_id * 2^jp outputs ahead of this one
        (mt_create_stream; this stream's pointer is put at 624 first)."""
        out = MT(0)
        self.L.or_mt_jump(self.h, int(jp), int(stream_id), out.h)
        return out
