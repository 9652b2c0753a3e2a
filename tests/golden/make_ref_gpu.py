#!/usr/bin/env python3
"""Generates ref_gpu.npz: the reference as it ships, run on a GPU.

For every structure of cases.py it loads the molecule through the reference's
own loader, sets it up as underdamped_ctrl does (alloc_GPU_arrays,
alloc_cudpp, setup_rng; sop.cu:133-140) and runs, from
oracle/_ref/libsopref_gpu.so:

  update_neighbor_list, update_pair_list   the CUDPP-based GPU list drivers
                                            (sop.cu:924-1262, 1452-1620; CUDPP
                                            by its stand-in, oracle/ref_cudpp_cub.cu)
  force_eval at `set temp 0`                the four force kernels and the
                                            (zero) cuRAND noise
                                            (energy.cu:81-150, 228-604)

and stores the lists (sorted pair keys for the 128-bead cases, SHA-256
digests and counts for the 4,000-bead ones) and the forces.  The extended
chains have an empty repulsive pair list at these cut-offs; the reference's
force_eval launches a zero-block grid there and exits (energy.cu:92-110),
so only their lists are stored.

Needs a GPU and the reference built into oracle/_ref (bash oracle/build_ref.sh
<reference tree>).  Each case runs in a process of its own (the reference
keeps its state in process globals).

Run from the repository root: python tests/golden/make_ref_gpu.py [--out PATH]
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
sys.path.insert(0, HERE)

import cases  # noqa: E402
from oracle import pyoracle as O  # noqa: E402


def one_case(name: str, out: str) -> None:
    R = O.ref_gpu_lib()
    mol, x, _, boxl = cases.build(name)
    res = {}
    with tempfile.TemporaryDirectory() as d:
        O.ref_load_molecule(R, mol, x, boxl, os.path.join(d, name))
    R.ref_set(b"temp", b"0")
    R.ref_device_setup(1234)
    lists = O.ref_lists(R)
    for which, (i, j, _) in lists.items():
        keys = cases.pair_keys(mol.n, i, j)
        res[f"{name}.{which}.count"] = np.int64(len(keys))
        if name in cases.SMALL:
            res[f"{name}.{which}"] = keys
        else:
            res[f"{name}.{which}.sha256"] = np.array(cases.digest(keys))
    if len(lists["pl_att"][0]) and len(lists["pl_rep"][0]):
        res[f"{name}.force"] = O.ref_forces(R, mol.n)
    np.savez_compressed(out, **res)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--case")
    ap.add_argument("--out", default=os.path.join(HERE, "ref_gpu.npz"))
    a = ap.parse_args()
    if a.case:
        one_case(a.case, a.out)
        return
    if not O.ref_gpu_available():
        sys.exit("oracle/_ref/libsopref_gpu.so is missing: run bash oracle/build_ref.sh <tree>")
    merged = {}
    with tempfile.TemporaryDirectory() as d:
        for name in cases.CASES:
            part = os.path.join(d, f"{name}.npz")
            subprocess.run([sys.executable, os.path.abspath(__file__), "--case", name,
                            "--out", part], check=True, stdout=subprocess.DEVNULL)
            with np.load(part) as z:
                merged.update({k: z[k] for k in z.files})
            print(name, "done", flush=True)
    np.savez_compressed(a.out, **merged)
    print("written", a.out)


if __name__ == "__main__":
    main()
