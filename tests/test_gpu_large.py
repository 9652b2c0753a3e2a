"""Parity at the large plain-path sizes, through the C ABI.

- 50,000 beads (per-contact epsilon in [0.7, 1.3]): neighbour and pair lists
  bit-exact as sets with the oracle's FP32 filters, forces within 1e-5 of
  FP64, on the same coordinates.
- 4,000 beads from the native structure and from a fully extended chain:
  the same checks every 1,000 steps of a running trajectory (lists rebuilt
  at the checkpoint's coordinates, forces without noise there).
"""
import numpy as np
import pytest

from helpers import att_sel, force_error, force_error_report, oracle_lists
from oracle import pyoracle as O
from sop_gb300 import engine, system

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5


def keys(i, j, n):
    """Pairs (i < j) as sorted int64 keys: set equality without Python sets."""
    a = np.minimum(i, j).astype(np.int64)
    b = np.maximum(i, j).astype(np.int64)
    return np.sort(a * n + b)


def check_lists_and_forces(e, mol, x, p, boxl):
    ai, aj, _ = e.list_pairs(0, 0)
    ri, rj, _ = e.list_pairs(0, 1)
    pai, paj, par = e.list_pairs(0, 2)
    pri, prj, _ = e.list_pairs(0, 3)
    nl_att, (nri, nrj), pl_att, (opi, opj) = oracle_lists(mol, x, p, boxl)
    n = mol.n
    np.testing.assert_array_equal(keys(ai, aj, n), keys(mol.nat_i[nl_att], mol.nat_j[nl_att], n))
    np.testing.assert_array_equal(keys(ri, rj, n), keys(nri, nrj, n))
    np.testing.assert_array_equal(keys(pai, paj, n), keys(mol.nat_i[pl_att], mol.nat_j[pl_att], n))
    np.testing.assert_array_equal(keys(pri, prj, n), keys(opi, opj, n))
    assert len(pri) > 0
    e.set_noise(np.zeros((n, 3), np.float32))
    e.force_eval()
    f = e.download()["force"]
    e.set_noise(None)
    fo, _ = O.forces_f64(mol, x, att_sel(mol, pai, paj), pri, prj)
    err = force_error(f, fo)
    rep = force_error_report(f, fo)
    print(n, rep)
    assert err <= FORCE_TOL, (err, rep)
    return len(ri), len(pri)


def test_50k_lists_bit_exact_and_forces():
    mol = system.generate(50000, 2, (0.7, 1.3))
    rng = np.random.default_rng(3)
    x = (mol.xyz + rng.normal(0.0, 0.25, mol.xyz.shape)).astype(np.float32)
    p = engine.baseline_params()
    with engine.plain(mol, x, p) as e:
        assert e.status(0)[0] == 0
        nnl, npl = check_lists_and_forces(e, mol, x, p, 500.0)
    assert nnl > 100 * mol.n and npl > 10 * mol.n   # 32 A / 16 A lists at this density


@pytest.mark.parametrize("start", ["native", "extended"])
def test_4000_checked_every_1000_steps(start):
    mol = system.generate(4000, 1)
    # the extended chain is 15,200 A long: a box that holds it without
    # self-images (at the default 500 A its periodic images would overlap)
    boxl = 500.0 if start == "native" else 40000.0
    p = engine.baseline_params(boxl=boxl)
    x0 = mol.xyz if start == "native" else mol.extended_xyz()
    with engine.plain(mol, x0, p, T=0.6) as e:
        for _ in range(3):
            e.step(1000)
            st, _ = e.status(0)
            assert st == 0
            x = e.download()["unc_pos"]
            e.update_neighbor_list()
            e.update_pair_list()
            check_lists_and_forces(e, mol, x, p, boxl)
