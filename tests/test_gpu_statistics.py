"""Long runs compared statistically with the reference algorithm.

The engine's noise is Philox; the reference draws cuRAND XORWOW
(energy.cu:588-604), so trajectories cannot match step for step.  Instead,
independent seeds of the 128-bead structure at kBT = 0.6 run on the GPU (one
batched context, one Philox stream each) and on the oracle's serial FP32 run
of the reference algorithm (orc_ref_*, its own generator per seed).  After an
equilibration, each trajectory's time averages of the total energy, Rg^2, the
native-contact fraction Q and the kinetic temperature are one sample; the two
sets of per-seed means must agree within 2 sigma of their combined standard
error.
"""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from helpers import oracle_lists
from oracle import pyoracle as O
from sop_gb300 import engine, system

pytestmark = pytest.mark.gpu

SEEDS = 16
EQUIL = 1000
SAMPLES = 40
EVERY = 100
T = 0.6
CUT = [0.0, 32.0, 0.0, 32.0, 0.0, 16.0, 0.0, 16.0]   # the engine's baseline cut-offs (A)


def gpu_means(mol):
    p = engine.baseline_params()
    e = engine.Engine(p)
    for k in range(SEEDS):
        e.add(mol, mol.xyz, T=T, traj=k)
    e.commit()
    e.step(EQUIL)
    acc = np.zeros((SEEDS, 4))
    for _ in range(SAMPLES):
        e.step(EVERY)
        for m in range(SEEDS):
            ob = e.observables(m)
            acc[m] += (e.energy(m)[4], ob["rgsq"], ob["Q"], ob["kinT"])
        assert all(e.status(m)[0] == 0 for m in range(SEEDS))
    e.close()
    return acc / SAMPLES


def ref_means(mol):
    p = engine.baseline_params()

    def one(k):
        r = O.RefRun(mol, mol.xyz, CUT, 0.05, 0.05, T, 50, 10, 9000 + k, k)
        r.advance(EQUIL)
        acc = np.zeros(4)
        for _ in range(SAMPLES):
            r.advance(EVERY)
            s = r.state()
            x, v = s["unc_pos"], s["vel"]
            nl_att, (nri, nrj), pl_att, (pri, prj) = oracle_lists(mol, x, p)
            _, en = O.forces_f64(mol, x, pl_att, pri, prj)
            ob = O.observables(mol, x, v)
            acc += (en.sum(), ob["rgsq"], ob["Q"], ob["kinT"])
        r.close()
        return acc / SAMPLES

    with ThreadPoolExecutor(8) as ex:
        return np.array(list(ex.map(one, range(SEEDS))))


def test_long_run_statistics_match_reference_within_2_sigma():
    mol = system.generate(128, 0)
    g = gpu_means(mol)
    r = ref_means(mol)
    names = ("energy", "rgsq", "Q", "kinT")
    for c, name in enumerate(names):
        mg, mr = g[:, c].mean(), r[:, c].mean()
        se = np.sqrt(g[:, c].var(ddof=1) / SEEDS + r[:, c].var(ddof=1) / SEEDS)
        assert abs(mg - mr) <= 2.0 * se, (name, mg, mr, se)
    # the comparison has power: the folded state is kept and T is reached
    assert g[:, 2].mean() > 0.6 and abs(g[:, 3].mean() - T) < 0.1
