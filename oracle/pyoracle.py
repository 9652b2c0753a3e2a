"""ctypes access to the oracle (oracle/liboracle.so) and to the reference's own
routines (oracle/_ref/libsopref.so: host routines and host list filters;
oracle/_ref/libsopref_gpu.so: the reference as it ships, list drivers and
force kernels on a GPU).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py -- never by the engine.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

# Force-field defaults of the reference (param.cpp:14-39, global.cpp:69-85, param.cpp:97)
DEFAULT_PARAMS = {"k_bnd": 20.0, "R0": 2.0, "eps_ss": 1.0, "sigma_ss": 3.5, "eps_rep": 1.0,
                  "boxl": 500.0, "rep6": 0}


def params_array(p: dict | None = None) -> np.ndarray:
    q = dict(DEFAULT_PARAMS)
    if p:
        q.update(p)
    return np.array([q["k_bnd"], q["R0"], q["eps_ss"], q["sigma_ss"], q["eps_rep"], q["boxl"],
                     q["rep6"]], np.float64)


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.orc_nl_rep.restype = ctypes.c_longlong
        L.orc_filter_rep.restype = ctypes.c_longlong
        L.orc_rcut2.restype = ctypes.c_float
        L.orc_rcut2.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_float]
        L.orc_ref_rgsq.restype = ctypes.c_double
        L.orc_ref_rgsq.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_double]
        _LIB = L
    return _LIB


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _i32(a):
    return np.ascontiguousarray(a, np.int32)


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


D = ctypes.c_double
LL = ctypes.c_longlong


def forces_f64(mol, x, att_sel, rep_i, rep_j, params=None, eps_energy=None):
    """FP64 forces (n, 3) and energy terms (bnd, ang_ss, vdw_att, vdw_rep) on the
    given pair lists.  att_sel indexes mol's native arrays."""
    x = _f32(x)
    att_sel = np.asarray(att_sel, np.int64)
    pai, paj = _i32(mol.nat_i[att_sel]), _i32(mol.nat_j[att_sel])
    pr0, pe = _f32(mol.nat_r0[att_sel]), _f32(mol.nat_eps[att_sel])
    pee = None if eps_energy is None else _f32(np.asarray(eps_energy)[att_sel])
    rep_i, rep_j = _i32(rep_i), _i32(rep_j)
    f = np.zeros((mol.n, 3), np.float64)
    e = np.zeros(4, np.float64)
    types = _i32(mol.types)
    lib().orc_forces_f64(mol.n, _p(x), _p(types), len(mol.bond_i), _p(_i32(mol.bond_i)),
                         _p(_i32(mol.bond_j)), _p(_f32(mol.bond_r0)), len(mol.ang_i),
                         _p(_i32(mol.ang_i)), _p(_i32(mol.ang_k)), len(pai), _p(pai), _p(paj),
                         _p(pr0), _p(pe), _p(pee), LL(len(rep_i)), _p(rep_i), _p(rep_j),
                         _p(params_array(params)), _p(f), _p(e))
    return f, e


def filter_att(mol, x, cand, fac, absval, boxl=500.0):
    """Indices of native contacts (from cand, or all when None) with d2 < rcut2."""
    x = _f32(x)
    ncand = len(mol.nat_i) if cand is None else len(cand)
    out = np.empty(max(ncand, 1), np.int32)
    sel = None if cand is None else _i32(cand)
    k = lib().orc_filter_att(_p(x), ncand, _p(sel), _p(_i32(mol.nat_i)), _p(_i32(mol.nat_j)),
                             _p(_f32(mol.nat_r0)), D(fac), D(absval), D(boxl), _p(out))
    return out[:k].copy()


def nl_rep(mol, x, fac, absval, boxl=500.0):
    """Repulsive neighbour list (i < j pairs) over the implicit master list."""
    x = _f32(x)
    cap = 1 << 16
    while True:
        oi = np.empty(cap, np.int32)
        oj = np.empty(cap, np.int32)
        k = lib().orc_nl_rep(mol.n, _p(x), _p(_i32(mol.types)), len(mol.nat_i),
                             _p(_i32(mol.nat_i)), _p(_i32(mol.nat_j)), D(fac), D(absval),
                             D(boxl), LL(cap), _p(oi), _p(oj))
        if k <= cap:
            return oi[:k].copy(), oj[:k].copy()
        cap = int(k)


def filter_rep(mol, x, ci, cj, fac, absval, boxl=500.0):
    x = _f32(x)
    ci, cj = _i32(ci), _i32(cj)
    oi = np.empty(max(len(ci), 1), np.int32)
    oj = np.empty(max(len(ci), 1), np.int32)
    k = lib().orc_filter_rep(_p(x), _p(_i32(mol.types)), LL(len(ci)), _p(ci), _p(cj), D(fac),
                             D(absval), D(boxl), _p(oi), _p(oj))
    return oi[:k].copy(), oj[:k].copy()


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, np.uint32)
    k = np.ascontiguousarray(key, np.uint32)
    out = np.empty(4, np.uint32)
    lib().orc_philox4x32_10(_p(c), _p(k), _p(out))
    return out


def noise_normals(n, step, traj, seed):
    out = np.empty((n, 3), np.float64)
    lib().orc_noise_normals(n, ctypes.c_ulonglong(step), ctypes.c_uint(traj),
                            ctypes.c_ulonglong(seed), _p(out))
    return out


def ref_gasdev(run_id: int, count: int) -> np.ndarray:
    """The reference's host Gaussian deviates after `set run` = run_id
    (random_generator.cpp:83-143, restated in orc_ref_gasdev)."""
    out = np.empty(count, np.float64)
    lib().orc_ref_gasdev(int(run_id), ctypes.c_longlong(count), _p(out))
    return out


def ref_rgsq(unc: np.ndarray, boxl: float) -> float:
    """Rg^2 of unwrapped coordinates as the reference computes it: the float
    pair sum of calculate_observables (sop.cu:563-580), restated in
    orc_ref_rgsq.  Thread-safe (ctypes releases the GIL), so a pool of
    threads can measure many frames at once."""
    x = np.ascontiguousarray(unc, np.float32)
    return lib().orc_ref_rgsq(int(x.shape[0]), x.ctypes.data, float(boxl))


def langevin_consts(h, zeta, T):
    out = np.empty(5, np.float64)
    lib().orc_langevin_consts(D(h), D(zeta), D(T), _p(out))
    return out


def observables(mol, x, v=None, boxl=500.0):
    out = np.empty(4, np.float64)
    x = _f32(x)
    vv = None if v is None else _f32(v)
    lib().orc_observables(mol.n, _p(x), _p(vv), len(mol.nat_i), _p(_i32(mol.nat_i)),
                          _p(_i32(mol.nat_j)), _p(_f32(mol.nat_r0)), D(boxl), _p(out))
    return {"Q": out[0], "rgsq": out[1], "kinT": out[2], "contct_nat": int(out[3])}


class RefRun:
    """The serial FP32 CPU baseline of one molecule (the reference's algorithm,
    orc_ref_* in sop_oracle.c); state persists between advance() calls.
    cut = [nl_att_fac, nl_att_abs, nl_rep_fac, nl_rep_abs, pl_att_fac, ...]."""

    def __init__(self, mol, unc, cut, h, zeta, T, nnlup, nplup, seed, traj, vel=None,
                 pos=None, params=None):
        L = lib()
        L.orc_ref_create.restype = ctypes.c_void_p
        L.orc_ref_advance.restype = ctypes.c_longlong
        L.orc_ref_advance.argtypes = [ctypes.c_void_p, ctypes.c_longlong]
        L.orc_ref_destroy.argtypes = [ctypes.c_void_p]
        L.orc_ref_state.argtypes = [ctypes.c_void_p] * 4
        self.n = mol.n
        keep = [_f32(unc), None if pos is None else _f32(pos), None if vel is None else _f32(vel),
                _i32(mol.types), _i32(mol.bond_i), _i32(mol.bond_j), _f32(mol.bond_r0),
                _i32(mol.ang_i), _i32(mol.ang_k), _i32(mol.nat_i), _i32(mol.nat_j),
                _f32(mol.nat_r0), _f32(mol.nat_eps), params_array(params),
                np.ascontiguousarray(cut, np.float64)]
        u, p, v, ty, bi, bj, br, ai, ak, ni, nj, nr, ne, pa, cu = keep
        self.h = L.orc_ref_create(
            mol.n, _p(u), _p(p), _p(v), _p(ty), len(bi), _p(bi), _p(bj), _p(br), len(ai),
            _p(ai), _p(ak), len(ni), _p(ni), _p(nj), _p(nr), _p(ne), _p(pa), _p(cu), D(h),
            D(zeta), D(T), nnlup, nplup, ctypes.c_ulonglong(seed), ctypes.c_uint(traj))
        if not self.h:
            raise MemoryError("orc_ref_create failed")

    def advance(self, nsteps: int) -> None:
        if lib().orc_ref_advance(self.h, nsteps) < 0:
            raise RuntimeError("orc_ref_advance failed")

    def state(self):
        out = [np.empty((self.n, 3), np.float32) for _ in range(3)]
        lib().orc_ref_state(self.h, *[_p(a) for a in out])
        return {"unc_pos": out[0], "pos": out[1], "vel": out[2]}

    def close(self):
        if self.h:
            lib().orc_ref_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


# ------------------------------------------------------ reference host routines
def ref_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libsopref.so"))


def ref_lib() -> ctypes.CDLL:
    global _REF
    if _REF is None:
        _REF = ctypes.CDLL(os.path.join(HERE, "_ref", "libsopref.so"))
        _bind_ref(_REF)
    return _REF


def ref_gpu_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libsopref_gpu.so"))


def ref_gpu_lib() -> ctypes.CDLL:
    """The reference as it ships (GPU list drivers, force kernels); a process
    loads either this library or ref_lib(), not both."""
    R = ctypes.CDLL(os.path.join(HERE, "_ref", "libsopref_gpu.so"))
    _bind_ref(R)
    return R


def _bind_ref(R) -> None:
    R.ref_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    R.ref_set.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    R.ref_device_setup.argtypes = [ctypes.c_ulonglong]


def ref_load_molecule(R, mol, x, boxl, prefix) -> None:
    """Writes mol (coordinates x) in the reference's file formats at prefix and
    runs the reference's loader on them (io.cpp:112-259) with `set boxl`."""
    from sop_gb300 import system
    system.write_reference_files(mol, prefix, x)
    R.ref_init_defaults()
    R.ref_set(b"boxl", repr(float(boxl)).encode())
    for k in ("bonds", "angles", "vdw", "init"):
        R.ref_load(k.encode(), f"{prefix}.{k}".encode())


def ref_lists(R) -> dict:
    """The reference's list drivers (update_neighbor_list then
    update_pair_list) on its current coordinates: 0-based (i, j) pairs of the
    attractive / repulsive neighbour and pair lists, r0 of the attractive ones."""
    c = np.zeros(4, np.int64)
    R.ref_update_lists(_p(c))
    out = {}
    for w, name in enumerate(("nl_att", "nl_rep", "pl_att", "pl_rep")):
        k = int(c[w])
        i = np.zeros(max(k, 1), np.int32)
        j = np.zeros(max(k, 1), np.int32)
        r = np.zeros(max(k, 1), np.float32)
        R.ref_list_copy(w, _p(i), _p(j), _p(r))
        out[name] = (i[:k].copy(), j[:k].copy(), r[:k].copy())
    return out


def ref_forces(R, n) -> np.ndarray:
    """force_eval of the reference on its current device pair lists."""
    f = np.zeros((n, 3), np.float32)
    R.ref_force_eval(_p(f))
    return f
