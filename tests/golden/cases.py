"""The structures the reference-made fixtures are computed on.

Shared by the fixture scripts in this directory (make_golden.py on the CPU,
make_ref_gpu.py on a GPU) and by the tests that read their output, so both
sides rebuild the same coordinates.

Every case is a molecule from the synthetic generator and a set of
coordinates: the native structure, the native structure with Gaussian noise
of 0.3 A on every coordinate ("perturbed"), or the fully extended chain
(beads 3.8 A apart on a line).  "two_types" marks a molecule whose beads are
of type 1 or 2: its native contacts are the pairs with |i-j| > 2 closer than
rcut_nat[ti][tj] (global.cpp:101-105), with the reference's per-type force
and energy coefficients (energy.cu:3-7, global.cpp:51-55).
"""
from __future__ import annotations

import hashlib

import numpy as np

from sop_gb300 import system

CASES = {
    "n128_native": dict(n=128, seed=0, start="native", boxl=500.0),
    "n128_perturbed": dict(n=128, seed=0, start="perturbed", boxl=500.0),
    "n128_extended": dict(n=128, seed=0, start="extended", boxl=500.0),
    "n128_two_types": dict(n=128, seed=3, start="perturbed", boxl=500.0, two_types=True),
    "n4000_native": dict(n=4000, seed=1, start="native", boxl=500.0),
    "n4000_perturbed": dict(n=4000, seed=1, start="perturbed", boxl=500.0),
    "n4000_extended": dict(n=4000, seed=1, start="extended", boxl=40000.0),
}
SMALL = [k for k, c in CASES.items() if c["n"] <= 128]

# force_coeff_att / -12 and coeff_att of the reference, by type pair
FORCE_EPS = np.array([[0.0, 0.0, 0.0], [0.0, 1.0, 0.8], [0.0, 0.8, 0.7]], np.float32)
ENERGY_EPS = np.array([[0.0, 0.0, 0.0], [0.0, 0.7, 0.8], [0.0, 0.8, 1.0]], np.float32)


def two_type_molecule(mol: system.Molecule, seed: int) -> system.Molecule:
    """The same chain with random bead types and natives chosen by type."""
    rng = np.random.default_rng(seed)
    types = rng.integers(1, 3, mol.n).astype(np.int32)
    ii, jj = np.triu_indices(mol.n, 3)
    x64 = mol.xyz.astype(np.float64)
    d = np.sqrt(((x64[jj] - x64[ii]) ** 2).sum(1)).astype(np.float32)
    cut = system.RCUT_NAT.astype(np.float32)[types[ii], types[jj]]
    nat = d < cut
    ni, nj, nr = ii[nat].astype(np.int32), jj[nat].astype(np.int32), d[nat]
    eps = FORCE_EPS[types[ni], types[nj]]
    return system.Molecule(mol.n, mol.xyz, mol.bond_i, mol.bond_j, mol.bond_r0, mol.ang_i,
                           mol.ang_j, mol.ang_k, mol.ang_r, ni, nj, nr, eps, types=types,
                           seed=mol.seed)


def build(name: str):
    """(molecule, coordinates, native energy epsilons, box) of a case.  The
    energy epsilons are the reference's coeff_att by type pair (0.7 for the
    all-type-1 molecules)."""
    c = CASES[name]
    mol = system.generate(c["n"], c["seed"])
    if c.get("two_types"):
        mol = two_type_molecule(mol, 7 + c["seed"])
    if c["start"] == "native":
        x = mol.xyz.copy()
    elif c["start"] == "perturbed":
        rng = np.random.default_rng(2024 + c["n"])
        x = (mol.xyz + rng.normal(0.0, 0.3, mol.xyz.shape)).astype(np.float32)
    else:
        x = mol.extended_xyz()
    eps_e = ENERGY_EPS[mol.types[mol.nat_i], mol.types[mol.nat_j]]
    return mol, np.ascontiguousarray(x, np.float32), eps_e, c["boxl"]


def pair_keys(n: int, i, j) -> np.ndarray:
    """Sorted uint32 keys min(i,j)*n + max(i,j): a list as a set."""
    i = np.asarray(i, np.int64)
    j = np.asarray(j, np.int64)
    return np.sort((np.minimum(i, j) * n + np.maximum(i, j)).astype(np.uint32))


def digest(keys: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(keys, np.uint32).tobytes()).hexdigest()
