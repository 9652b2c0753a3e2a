"""Molecule topology, the synthetic generator and the reference's file formats.

A :class:`Molecule` holds what the reference's four data files hold
(io.cpp:112-259): bonds with native lengths, i,i+2 angles, native contacts
with native distances (and, beyond the reference, a per-contact epsilon), the
implicit non-native (repulsive) set, per-bead types and coordinates.

Indices are 0-based here; the reference files are 1-based and the readers and
writers convert.  The non-native set is implicit: every pair with |i-j| > 2
that is not a native contact -- exactly what the reference's vdw file lists as
its repulsive master list (io.cpp:216-225).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_GEN = None


def _gen_lib() -> ctypes.CDLL:
    global _GEN
    if _GEN is None:
        path = os.path.join(_HERE, "libsopgen.so")
        if not os.path.exists(path):
            raise RuntimeError(
                f"{path} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
        lib = ctypes.CDLL(path)
        P = ctypes.c_void_p
        lib.sopgen_create.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_double,
                                      ctypes.c_double, ctypes.POINTER(P)]
        lib.sopgen_destroy.argtypes = [P]
        lib.sopgen_counts.argtypes = [P] + [ctypes.POINTER(ctypes.c_int)] * 4
        for name in ("sopgen_native_xyz", "sopgen_bonds", "sopgen_angles", "sopgen_natives"):
            getattr(lib, name).restype = ctypes.c_int
        lib.sopgen_extended_xyz.argtypes = [ctypes.c_int, P]
        lib.sopgen_ensemble.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                        P, P]
        lib.sopgen_requests.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                        ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                        P, P, P, P, P]
        _GEN = lib
    return _GEN


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


@dataclass
class Molecule:
    """One SOP molecule (0-based indices)."""
    n: int
    xyz: np.ndarray                      # (n, 3) float32 native coordinates
    bond_i: np.ndarray                   # (B,) int32
    bond_j: np.ndarray
    bond_r0: np.ndarray                  # (B,) float32
    ang_i: np.ndarray                    # (A,) int32, soft sphere acts on (i, k)
    ang_j: np.ndarray
    ang_k: np.ndarray
    ang_r: np.ndarray                    # (A,) float32 native i..k distance
    nat_i: np.ndarray                    # (C,) int32, i < j, sorted by (i, j)
    nat_j: np.ndarray
    nat_r0: np.ndarray                   # (C,) float32
    nat_eps: np.ndarray                  # (C,) float32, epsilon used by the force
    types: np.ndarray = field(default=None)  # (n,) int32 in {1, 2}; None -> all 1
    seed: int = 0

    def __post_init__(self):
        if self.types is None:
            self.types = np.ones(self.n, np.int32)

    @property
    def n_rep_master(self) -> int:
        """Size of the implicit non-native master list."""
        n = self.n
        pairs = (n - 3) * (n - 2) // 2 if n > 3 else 0
        return pairs - len(self.nat_i)

    def extended_xyz(self) -> np.ndarray:
        """Beads on the x axis 3.8 A apart, centred on the origin."""
        out = np.empty((self.n, 3), np.float32)
        _gen_lib().sopgen_extended_xyz(self.n, _ptr(out))
        return out


def generate(n: int, seed: int, eps_range: tuple[float, float] | None = None) -> Molecule:
    """Synthetic native structure of n beads (deterministic in `seed`).

    eps_range=(lo, hi) draws a per-contact epsilon uniform in [lo, hi];
    None gives every native contact epsilon 1.0.
    """
    lib = _gen_lib()
    lo, hi = (1.0, 1.0) if eps_range is None else eps_range
    h = ctypes.c_void_p()
    rc = lib.sopgen_create(int(n), int(seed) & (2**64 - 1), float(lo), float(hi), ctypes.byref(h))
    if rc != 0:
        raise RuntimeError(f"sopgen_create(n={n}, seed={seed}) failed with {rc}")
    try:
        cnt = [ctypes.c_int() for _ in range(4)]
        lib.sopgen_counts(h, *[ctypes.byref(c) for c in cnt])
        nb, B, A, C = (c.value for c in cnt)
        xyz = np.empty((nb, 3), np.float32)
        lib.sopgen_native_xyz(h, _ptr(xyz))
        bi, bj = np.empty(B, np.int32), np.empty(B, np.int32)
        br = np.empty(B, np.float32)
        lib.sopgen_bonds(h, _ptr(bi), _ptr(bj), _ptr(br))
        ai, aj, ak = (np.empty(A, np.int32) for _ in range(3))
        ar = np.empty(A, np.float32)
        lib.sopgen_angles(h, _ptr(ai), _ptr(aj), _ptr(ak), _ptr(ar))
        ni, nj = np.empty(C, np.int32), np.empty(C, np.int32)
        nr, ne = np.empty(C, np.float32), np.empty(C, np.float32)
        lib.sopgen_natives(h, _ptr(ni), _ptr(nj), _ptr(nr), _ptr(ne))
    finally:
        lib.sopgen_destroy(h)
    return Molecule(nb, xyz, bi, bj, br, ai, aj, ak, ar, ni, nj, nr, ne, seed=seed)


def ensemble_spec(count: int, n_lo: int, n_hi: int, t_lo: float, t_hi: float,
                  seed: int) -> tuple[np.ndarray, np.ndarray]:
    """Sizes (log-uniform) and temperatures (uniform) of a batched ensemble."""
    ns = np.empty(count, np.int32)
    ts = np.empty(count, np.float32)
    rc = _gen_lib().sopgen_ensemble(count, n_lo, n_hi, t_lo, t_hi, seed, _ptr(ns), _ptr(ts))
    if rc:
        raise ValueError("bad ensemble specification")
    return ns, ts


def request_stream(rate: float, duration: float, n_range=(50, 20000), step_range=(1e4, 1e6),
                   t_range=(0.5, 0.8), seed: int = 5, cap: int = 1 << 20) -> dict:
    """A Poisson request stream of folding (native start) / unfolding (extended start) jobs."""
    arr = np.empty(cap, np.float64)
    ns = np.empty(cap, np.int32)
    st = np.empty(cap, np.int64)
    ts = np.empty(cap, np.float32)
    ext = np.empty(cap, np.int32)
    cnt = ctypes.c_int()
    rc = _gen_lib().sopgen_requests(rate, duration, n_range[0], n_range[1], step_range[0],
                                    step_range[1], t_range[0], t_range[1], seed, cap,
                                    ctypes.byref(cnt), _ptr(arr), _ptr(ns), _ptr(st), _ptr(ts),
                                    _ptr(ext))
    if rc:
        raise ValueError("bad request-stream specification")
    k = cnt.value
    return {"arrival": arr[:k].copy(), "n": ns[:k].copy(), "steps": st[:k].copy(),
            "T": ts[:k].copy(), "extended": ext[:k].copy()}


# ------------------------------------------------------------------ file formats
# rcut_nat[itype][jtype] (global.cpp:101-105): a vdw-file pair is native iff
# its distance is below this.
RCUT_NAT = np.array([[0.0, 0.0, 0.0], [0.0, 8.0, 11.0], [0.0, 11.0, 14.0]])


def write_reference_files(mol: Molecule, prefix: str, xyz: np.ndarray | None = None) -> dict:
    """Writes <prefix>.bonds/.angles/.vdw/.init in the reference's formats.

    The vdw file lists natives and the full non-native master list with their
    native distances and types (io.cpp:174-230); it is O(N^2) lines, so this
    is meant for small molecules.
    """
    xyz = mol.xyz if xyz is None else xyz
    paths = {k: f"{prefix}.{k}" for k in ("bonds", "angles", "vdw", "init")}
    with open(paths["bonds"], "w") as f:
        f.write(f"bonds {len(mol.bond_i)}\n")
        for i, j, r in zip(mol.bond_i, mol.bond_j, mol.bond_r0):
            f.write(f"{i + 1} {j + 1} {float(r):.9g}\n")
    with open(paths["angles"], "w") as f:
        f.write(f"angles {len(mol.ang_i)}\n")
        for i, j, k, r in zip(mol.ang_i, mol.ang_j, mol.ang_k, mol.ang_r):
            f.write(f"{i + 1} {j + 1} {k + 1} {float(r):.9g}\n")
    nat = set(zip(mol.nat_i.tolist(), mol.nat_j.tolist()))
    rep_i, rep_j = rep_master(mol)
    x64 = mol.xyz.astype(np.float64)
    with open(paths["vdw"], "w") as f:
        f.write(f"natives {len(mol.nat_i)} nonnatives {len(rep_i)}\n")
        for i, j, r in zip(mol.nat_i, mol.nat_j, mol.nat_r0):
            f.write(f"{i + 1} {j + 1} {float(r):.9g} {mol.types[i]} {mol.types[j]}\n")
        d = np.sqrt(((x64[rep_j] - x64[rep_i]) ** 2).sum(1)).astype(np.float32)
        for i, j, r in zip(rep_i, rep_j, d):
            assert (int(i), int(j)) not in nat
            f.write(f"{i + 1} {j + 1} {float(r):.9g} {mol.types[i]} {mol.types[j]}\n")
    with open(paths["init"], "w") as f:
        f.write(f"init {mol.n}\n")
        for i in range(mol.n):
            f.write(f"{i + 1} {xyz[i, 0]:.9g} {xyz[i, 1]:.9g} {xyz[i, 2]:.9g}\n")
    return paths


def rep_master(mol: Molecule) -> tuple[np.ndarray, np.ndarray]:
    """The implicit non-native master list as explicit (i, j), i < j, (i, j)-sorted."""
    n = mol.n
    ii, jj = np.triu_indices(n, 3)
    ii = ii.astype(np.int32)
    jj = jj.astype(np.int32)
    if len(mol.nat_i):
        key = ii.astype(np.int64) * n + jj
        nkey = mol.nat_i.astype(np.int64) * n + mol.nat_j
        keep = ~np.isin(key, nkey)
        ii, jj = ii[keep], jj[keep]
    return ii, jj


def read_reference_files(bonds: str, angles: str, vdw: str, init: str) -> Molecule:
    """Reads the reference's four data files (io.cpp:126-257).

    The vdw file's non-native pairs must be the complement of its natives over
    |i-j| > 2 with consistent per-bead types; that is the content the
    reference's SOP inputs carry, and the engine keeps it implicit.
    """
    def _lines(path):
        with open(path) as f:
            return [ln.split() for ln in f.read().splitlines()]

    bl = _lines(bonds)
    nb = int(bl[0][1])
    b = np.array([[float(t) for t in ln[:3]] for ln in bl[1:1 + nb]]).reshape(-1, 3)
    al = _lines(angles)
    na = int(al[0][1])
    a = np.array([[float(t) for t in ln[:4]] for ln in al[1:1 + na]]).reshape(-1, 4)
    vl = _lines(vdw)
    ncon = int(vl[0][1]) + int(vl[0][3])
    v = vl[1:1 + ncon]
    il = _lines(init)
    n = int(il[0][1])
    xyz = np.array([[float(t) for t in ln[1:4]] for ln in il[1:1 + n]], np.float32)
    types = np.zeros(n + 1, np.int32)
    nat = []
    nrep = 0
    for ln in v:
        i, j, r, ti, tj = int(ln[0]), int(ln[1]), np.float32(float(ln[2])), int(ln[3]), int(ln[4])
        for bead, t in ((i, ti), (j, tj)):
            if types[bead] not in (0, t):
                raise ValueError(f"bead {bead} has inconsistent types in {vdw}")
            types[bead] = t
        if r < RCUT_NAT[ti][tj]:
            lo, hi = min(i, j), max(i, j)
            nat.append((lo - 1, hi - 1, r))
        else:
            nrep += 1
    types = types[1:]
    types[types == 0] = 1
    nat.sort()
    ni = np.array([t[0] for t in nat], np.int32)
    nj = np.array([t[1] for t in nat], np.int32)
    nr = np.array([t[2] for t in nat], np.float32)
    mol = Molecule(n, xyz, b[:, 0].astype(np.int32) - 1, b[:, 1].astype(np.int32) - 1,
                   b[:, 2].astype(np.float32), a[:, 0].astype(np.int32) - 1,
                   a[:, 1].astype(np.int32) - 1, a[:, 2].astype(np.int32) - 1,
                   a[:, 3].astype(np.float32), ni, nj, nr, np.ones(len(ni), np.float32),
                   types=types)
    if nrep != mol.n_rep_master:
        raise ValueError(f"{vdw}: {nrep} non-native pairs, expected the complement "
                         f"({mol.n_rep_master}) of the natives over |i-j| > 2")
    return mol
