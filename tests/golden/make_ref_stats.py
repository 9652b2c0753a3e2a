#!/usr/bin/env python3
"""Generates ref_stats.npz: long-run statistics of the reference program.

The reference program itself (oracle/_ref/sop2ref.x: main() and
underdamped_ctrl of sop.cu, built by oracle/build_ref.sh) runs its own input
script on each structure once per seed:

  set run R; set dynamics underdamped; set temp T; set zeta 0.05; set t_step 0.05;
  set nstep 5000; set nup 100; set nnlup 50; set cutofftype neighborlist;
  set boxl 500; load bonds|angles|vdw|init <files>; run;

so the neighbour list is rebuilt every 50 steps and the pair list every step
(sop.cu:197-243), cut-offs 3.2 / 2.5 x r0 or sigma, cuRAND noise.  The
reference seeds cuRAND with the constant 1234 (sop.cu:139); the build wraps
setup_rng so that SOP_REF_CURAND_SEED replaces it (oracle/ref_link_wraps.cpp),
and each run gets its own seed.  The progress file the reference writes every
nup steps (sop.cu:252-262) gives, after EQUIL steps, SAMPLES rows per run:
rna_etot (its native energy uses coeff_att, 0.7 for type (1, 1)), Rg^2, Q and
the kinetic temperature.  Their per-run means are stored, one row per seed.

Cases: the 128-bead structure (seed 0, 256 runs) and the 4,000-bead
structure (seed 1, 144 runs: 48, then 96 more with --append), both from the
native structure at kBT = 0.6.  A fully extended start
cannot run in the reference at these cut-offs: its repulsive pair list is
empty and force_eval exits on the zero-block launch (energy.cu:92-110).

Needs a GPU.  Run from the repository root:
python tests/golden/make_ref_stats.py [--out PATH] [--jobs J] [--cases n128,n4000]
    [--runs R --append]   (R more runs of the given cases, appended to PATH)
"""
import argparse
import os
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from sop_gb300 import system  # noqa: E402

EXE = os.path.join(ROOT, "oracle", "_ref", "sop2ref.x")
# the same program built with its host noise generator (--rng host):
# gasdev of random_generator.cpp seeded by `set run`, in place of cuRAND
EXE_HOST = os.path.join(ROOT, "oracle", "_ref", "sop2ref_hostrng.x")
T = 0.6
NSTEP, NUP, NNLUP, EQUIL = 5000, 100, 50, 1000
# setup_rng seeds bead i's XORWOW generator with seed + i (GPUvars.cu:417-425);
# run k takes seed base + k * SEED_STRIDE, so no two runs share a generator
SEED_STRIDE = 1_000_003
STATS_CASES = {"n128": dict(n=128, seed=0, runs=256, base=1_000_000),
               "n4000": dict(n=4000, seed=1, runs=48, base=900_000_000)}


SCRIPT = """set run {run};
set dynamics underdamped;
set temp {T};
set zeta 0.05;
set t_step 0.05;
set nstep {nstep};
set nup {nup};
set nnlup {nnlup};
set cutofftype neighborlist;
set boxl 500;
load bonds {p}.bonds;
load angles {p}.angles;
load vdw {p}.vdw;
load init {p}.init;
run;
"""


def run_one(prefix: str, seed: int, workroot: str, exe: str = EXE) -> np.ndarray:
    d = tempfile.mkdtemp(dir=workroot)
    with open(os.path.join(d, "input"), "w") as f:
        # `set run` seeds the host generator (param.cpp:274-279): runs stay
        # distinct whichever noise path the program was built with
        f.write(SCRIPT.format(T=T, nstep=NSTEP, nup=NUP, nnlup=NNLUP, p=prefix,
                              run=seed % 1_000_000_007))
    env = dict(os.environ, SOP_REF_CURAND_SEED=str(seed))
    subprocess.run([exe, "input"], cwd=d, env=env, check=True, stdout=subprocess.DEVNULL,
                   stderr=subprocess.DEVNULL)
    rows = []
    with open(os.path.join(d, "update.out")) as f:
        for line in f:
            t = line.split()
            istep = float(t[0])
            if istep > EQUIL:
                # istep T kinT e_bnd e_ang_ss e_att e_rep e_vdw rna_etot Q contct_nat rgsq
                rows.append((float(t[8]), float(t[11]), float(t[9]), float(t[2])))
    subprocess.run(["rm", "-rf", d], check=True)
    a = np.array(rows)
    if len(a) != (NSTEP - EQUIL) // NUP:
        raise RuntimeError(f"seed {seed}: {len(a)} samples in {d}")
    return a.mean(axis=0)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "ref_stats.npz"))
    ap.add_argument("--jobs", type=int, default=min(12, os.cpu_count() or 4))
    ap.add_argument("--cases", default=",".join(STATS_CASES))
    ap.add_argument("--runs", type=int, default=0, help="runs per case (0: the case's own count)")
    ap.add_argument("--append", action="store_true",
                    help="add the runs to those already in --out, with the next seeds")
    ap.add_argument("--rng", choices=["curand", "host"], default="curand",
                    help="noise path of the reference program (host: its gasdev generator)")
    a = ap.parse_args()
    exe = EXE if a.rng == "curand" else EXE_HOST
    if not os.path.exists(exe):
        sys.exit(f"{exe} is missing: run bash oracle/build_ref.sh <reference tree>")
    out = {"T": np.float64(T), "nstep": np.int64(NSTEP), "nup": np.int64(NUP),
           "nnlup": np.int64(NNLUP), "equil": np.int64(EQUIL),
           "columns": np.array(["rna_etot", "rgsq", "Q", "kinT"])}
    old = {}
    if a.append and os.path.exists(a.out):
        with np.load(a.out) as z:
            old = {k: z[k] for k in z.files}
        out.update(old)
    with tempfile.TemporaryDirectory() as work:
        for name in a.cases.split(","):
            c = STATS_CASES[name]
            mol = system.generate(c["n"], c["seed"])
            prefix = os.path.join(work, name)
            system.write_reference_files(mol, prefix)
            first = len(old.get(f"{name}.seeds", []))
            runs = a.runs or c["runs"]
            seeds = [c["base"] + k * SEED_STRIDE for k in range(first, first + runs)]
            with ThreadPoolExecutor(a.jobs) as ex:
                means = list(ex.map(lambda s: run_one(prefix, s, work, exe), seeds))
            if first:
                means = list(old[f"{name}.means"]) + means
                seeds = list(old[f"{name}.seeds"]) + seeds
            out[f"{name}.means"] = np.array(means)
            out[f"{name}.seeds"] = np.array(seeds, np.int64)
            print(name, "mean over runs", np.array(means).mean(axis=0), flush=True)
    np.savez_compressed(a.out, **out)
    print("written", a.out)


if __name__ == "__main__":
    main()
