"""The drop-in, end to end: the reference program run over the engine.

sop_gb300/shim/build_shim_ref.sh links the reference's own objects (parser,
loaders, host energies, observables, writers, underdamped_ctrl) with
sop_gb300_shim.cu and libsopgpu.so.  The reference's input script runs 1,000
steps; every 100 steps its loop reads the state back (sop.cu:252-263) and
writes a progress line from its own energy_eval and calculate_observables
(sop.cu:256-259), while the shim logs the engine's own energy terms and
observables for the same state.  The two must agree: the reference's FP32
host sums against the engine's FP32 terms with FP64 sums, written with 6
decimals.  The two-type molecule checks that the shim hands the engine the
reference's per-type native force and energy coefficients (energy.cu:3-7,
global.cpp:51-55).

Needs the reference's source tree (SOP_REFERENCE_DIR) to build the linked
program; skipped without it.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from sop_gb300 import system

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import cases  # noqa: E402

SCRIPT = """set dynamics underdamped;
set temp 0.6;
set zeta 0.05;
set t_step 0.05;
set nstep 1000;
set nup 100;
set nnlup 50;
set cutofftype neighborlist;
set boxl 500;
load bonds {p}.bonds;
load angles {p}.angles;
load vdw {p}.vdw;
load init {p}.init;
run;
"""


@pytest.fixture(scope="module")
def dropin_exe():
    ref = os.environ.get("SOP_REFERENCE_DIR", "")
    if not ref or not os.path.exists(os.path.join(ref, "global.h")):
        pytest.skip("SOP_REFERENCE_DIR does not name a reference source tree")
    subprocess.run(["bash", os.path.join(ROOT, "sop_gb300", "shim", "build_shim_ref.sh"), ref],
                   check=True, capture_output=True)
    return os.path.join(ROOT, "sop_gb300", "shim", "_build", "sop2_gb300.x")


@pytest.mark.parametrize("two_types", [False, True])
def test_reference_loop_over_engine(dropin_exe, tmp_path, two_types):
    mol = system.generate(128, 3 if two_types else 0)
    if two_types:
        mol = cases.two_type_molecule(mol, 10)
    prefix = str(tmp_path / "m")
    system.write_reference_files(mol, prefix)
    (tmp_path / "input").write_text(SCRIPT.format(p=prefix))
    check = tmp_path / "engine.log"
    env = dict(os.environ, SOP_SHIM_CHECK_FILE=str(check))
    r = subprocess.run([dropin_exe, "input"], cwd=tmp_path, env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    ref = np.loadtxt(tmp_path / "update.out", ndmin=2)
    eng = np.loadtxt(check, ndmin=2)
    assert len(ref) == len(eng) == 10
    # update.out: istep T kinT e_bnd e_ang_ss e_att e_rep e_vdw rna_etot Q contct_nat rgsq
    # engine.log: step e_bnd e_ang_ss e_att e_rep rna_etot Q rgsq kinT contct_nat
    np.testing.assert_array_equal(ref[:, 0], eng[:, 0])
    for rc, ec in ((3, 1), (4, 2), (5, 3), (6, 4), (8, 5)):
        np.testing.assert_allclose(ref[:, rc], eng[:, ec], rtol=2e-5, atol=2e-6)
    np.testing.assert_array_equal(ref[:, 10], eng[:, 9])          # native contacts
    np.testing.assert_allclose(ref[:, 9], eng[:, 6], atol=1e-6)   # Q
    np.testing.assert_allclose(ref[:, 11], eng[:, 7], rtol=1e-5)  # Rg^2
    np.testing.assert_allclose(ref[:, 2], eng[:, 8], rtol=1e-5)   # kinetic T
    # the run stayed finite and warm (and folded, for the generator's own
    # molecule; the two-type molecule's native set is not the generator's)
    assert np.isfinite(ref).all() and 0.3 < ref[5:, 2].mean() < 0.9
    if not two_types:
        assert ref[:, 9].min() > 0.6
