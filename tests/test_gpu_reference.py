"""The engine against the reference's own outputs on the same coordinates.

Fixtures (tests/golden): ref_lists.npz from the reference's host list
filters (sop.cu:1351-1448, 1707-1823) and ref_gpu.npz from the reference as
it ships, run on a GPU: its CUDPP-based list drivers and its force kernels
(force_eval at T = 0, energy.cu:81-150, 228-584).  The engine runs in the
reference's factor mode (3.2 / 2.5 x r0 or sigma).

- lists: bit-exact as sets, every case (native, perturbed, extended, two
  bead types; 128 and 4,000 beads);
- forces: the engine against the reference's kernels within the reference's
  own FP32 error (the bounds its kernels keep against FP64:
  test_golden.assert_force_close_to_reference), and against FP64 within 1e-5.
"""
import os
import sys

import numpy as np
import pytest

from helpers import att_sel, force_error
from oracle import pyoracle as O
from sop_gb300 import engine

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLD)
import cases  # noqa: E402
from test_golden import assert_force_close_to_reference, assert_lists_equal  # noqa: E402


def engine_for(name):
    mol, x, eps_e, boxl = cases.build(name)
    p = engine.default_params(h=0.05, zeta=0.05, boxl=boxl)
    e = engine.plain(mol, x, p, T=0.6, eps_energy=eps_e)
    return e, mol, x, boxl


@pytest.mark.parametrize("name", list(cases.CASES))
def test_engine_lists_match_reference(name):
    e, mol, x, _ = engine_for(name)
    with e:
        lists = {}
        for which, w in (("nl_att", 0), ("nl_rep", 1), ("pl_att", 2), ("pl_rep", 3)):
            i, j, _ = e.list_pairs(0, w)
            lists[which] = cases.pair_keys(mol.n, i, j)
    assert_lists_equal(np.load(os.path.join(GOLD, "ref_lists.npz")), name, lists)
    gpath = os.path.join(GOLD, "ref_gpu.npz")
    if os.path.exists(gpath):
        assert_lists_equal(np.load(gpath), name, lists)


@pytest.mark.parametrize("name", [k for k, c in cases.CASES.items() if c["start"] != "extended"])
def test_engine_forces_match_reference_kernels(name):
    gpath = os.path.join(GOLD, "ref_gpu.npz")
    if not os.path.exists(gpath):
        pytest.skip("ref_gpu.npz not generated")
    f_ref = np.load(gpath)[f"{name}.force"]
    e, mol, x, boxl = engine_for(name)
    with e:
        e.set_noise(np.zeros((mol.n, 3), np.float32))
        e.force_eval()
        f = e.download()["force"]
        ai, aj, _ = e.list_pairs(0, 2)
        ri, rj, _ = e.list_pairs(0, 3)
    f64, _ = O.forces_f64(mol, x, att_sel(mol, ai, aj), ri, rj, params={"boxl": boxl})
    err64 = force_error(f, f64)
    print(name, "engine vs reference kernels:", force_error(f, f_ref), "engine vs FP64:", err64)
    assert_force_close_to_reference(name, f, f_ref)
    assert err64 <= 1e-5, (name, err64)
