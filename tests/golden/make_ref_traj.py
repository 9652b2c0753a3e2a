#!/usr/bin/env python3
"""Generates ref_traj.npz: trajectories of the reference program with known noise.

The reference program built with its host noise generator
(oracle/_ref/sop2ref_hostrng.x: USE_CURAND taken back, so random_force draws
var * gasdev() per bead and component, energy.cu:168-188) runs its own input
script with `set run 7` and `set nup 1`, and its trajectory writer
(record_traj, io.cpp:261-282) records the unwrapped coordinates after every
step.  The noise sequence is then known: the generator's deviates after
`set run 7` in order, 3 per bead per force evaluation (the set-up's first,
then one per step), which the oracle restates bit for bit (orc_ref_gasdev).

Cases (reference settings: factor-mode cut-offs, neighbour list every 50
steps, pair list every step, kBT 0.6, h = zeta = 0.05, box 500 A, native
start): the 128-bead structure (seed 0), frames after steps 1-10, 20, 30, 50,
100, 150, 200, 300; the 4,000-bead structure (seed 1), frames after steps 1,
10, 50, 100.  Coordinates are the writer's %f values.

Needs a GPU and the reference built into oracle/_ref.  Run from the
repository root: python tests/golden/make_ref_traj.py [--out PATH]
"""
import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from sop_gb300 import system  # noqa: E402

EXE = os.path.join(ROOT, "oracle", "_ref", "sop2ref_hostrng.x")
RUN = 7
CASES = {"n128": dict(n=128, seed=0, frames=[*range(1, 11), 20, 30, 50, 100, 150, 200, 300]),
         "n4000": dict(n=4000, seed=1, frames=[1, 10, 50, 100])}
SCRIPT = """set run {run};
set dynamics underdamped;
set temp 0.6;
set zeta 0.05;
set t_step 0.05;
set nstep {nstep};
set nup 1;
set nnlup 50;
set cutofftype neighborlist;
set boxl 500;
load bonds {p}.bonds;
load angles {p}.angles;
load vdw {p}.vdw;
load init {p}.init;
run;
"""


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "ref_traj.npz"))
    a = ap.parse_args()
    if not os.path.exists(EXE):
        sys.exit(f"{EXE} is missing: run bash oracle/build_ref.sh <reference tree>")
    out = {"run": np.int64(RUN)}
    for name, c in CASES.items():
        with tempfile.TemporaryDirectory() as d:
            system.write_reference_files(system.generate(c["n"], c["seed"]), os.path.join(d, "m"))
            with open(os.path.join(d, "input"), "w") as f:
                f.write(SCRIPT.format(run=RUN, nstep=max(c["frames"]), p=os.path.join(d, "m")))
            subprocess.run([EXE, "input"], cwd=d, check=True, stdout=subprocess.DEVNULL)
            # frame 0 is the set-up's (record_traj before the loop, sop.cu:191-194)
            fr = np.loadtxt(os.path.join(d, "traj_uncorrected.bin")).reshape(-1, c["n"], 3)
        out[f"{name}.steps"] = np.array(c["frames"], np.int64)
        out[f"{name}.unc"] = fr[c["frames"]].astype(np.float32)
        print(name, fr.shape, flush=True)
    np.savez_compressed(a.out, **out)
    print("written", a.out)


if __name__ == "__main__":
    main()
