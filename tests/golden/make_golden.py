#!/usr/bin/env python3
"""Generates the golden fixtures in this directory from the reference's own
host routines (oracle/_ref/libsopref.so, built by oracle/build_ref.sh from the
reference's unmodified sources).

Fixtures:
  m64.{bonds,angles,vdw,init}  a 64-bead synthetic molecule (seed 11) in the
                               reference's file formats
  m64_load.npz                 what the reference's loader (io.cpp:112-259)
                               parsed from those files
  m128_energy.npz              perturbed 128-bead coordinates (seed 0), pair
                               lists, and the reference's FP32 host energies
                               (energy.cu:194-225, 278-307, 369-442) and
                               observables (sop.cu:528-611) on them, for the
                               factor-mode and absolute-mode lists
  m128_out.{traj,traj_unc,coord,unccoord,vel}
                               the reference's output writers (io.cpp:261-381)
                               on that state (wrapped = unwrapped coordinates)
  m128_update.txt              its progress line for step 1000 (sop.cu:256-259)

Run from the repository root: python tests/golden/make_golden.py
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle as O  # noqa: E402
from sop_gb300 import system  # noqa: E402


def P(a):
    return ctypes.c_void_p(a.ctypes.data)


def reference_load(R, prefix):
    R.ref_init_defaults()
    for k in ("bonds", "angles", "vdw", "init"):
        R.ref_load(k.encode(), f"{prefix}.{k}".encode())
    sz = np.zeros(7, np.int32)
    R.ref_sizes(P(sz))
    nbead, nbnd, nang, natt, nrep = (int(v) for v in sz[:5])
    out = {k: np.zeros(n, t) for k, n, t in [
        ("bi", nbnd, np.int32), ("bj", nbnd, np.int32), ("br0", nbnd, np.float32),
        ("ai", nang, np.int32), ("ak", nang, np.int32),
        ("ni", natt, np.int32), ("nj", natt, np.int32), ("nti", natt, np.int32),
        ("ntj", natt, np.int32), ("nr0", natt, np.float32),
        ("ri", nrep, np.int32), ("rj", nrep, np.int32), ("rti", nrep, np.int32),
        ("rtj", nrep, np.int32)]}
    R.ref_topology(*[P(out[k]) for k in ("bi", "bj", "br0", "ai", "ak", "ni", "nj", "nti", "ntj",
                                         "nr0", "ri", "rj", "rti", "rtj")])
    pos = np.zeros((nbead, 3), np.float32)
    unc = np.zeros((nbead, 3), np.float32)
    R.ref_positions(P(pos), P(unc))
    out.update(pos=pos, unc=unc, sizes=sz)
    return out


def main():
    if not O.ref_available():
        sys.exit("oracle/_ref/libsopref.so is missing: run bash oracle/build_ref.sh")
    R = O.ref_lib()

    m64 = system.generate(64, 11)
    prefix = os.path.join(HERE, "m64")
    system.write_reference_files(m64, prefix)
    np.savez_compressed(os.path.join(HERE, "m64_load.npz"), **reference_load(R, prefix))

    m = system.generate(128, 0)
    tmp = os.path.join(HERE, "_m128_tmp")
    system.write_reference_files(m, tmp)
    reference_load(R, tmp)
    for k in ("bonds", "angles", "vdw", "init"):
        os.remove(f"{tmp}.{k}")
    rng = np.random.default_rng(2024)
    x = (m.xyz + rng.normal(0.0, 0.3, m.xyz.shape)).astype(np.float32)
    v = rng.normal(0.0, 0.8, m.xyz.shape).astype(np.float32)
    R.ref_set_state(P(x), P(v))
    fx = {}
    for mode, (nlf, nla, plf, pla) in {"factor": (3.2, 0.0, 2.5, 0.0),
                                       "absolute": (0.0, 32.0, 0.0, 16.0)}.items():
        att = O.filter_att(m, x, None, nlf, nla)
        ri, rj = O.nl_rep(m, x, nlf, nla)
        patt = O.filter_att(m, x, att, plf, pla)
        pri, prj = O.filter_rep(m, x, ri, rj, plf, pla)
        ai = np.ascontiguousarray(m.nat_i[patt]).astype(np.int32)
        aj = np.ascontiguousarray(m.nat_j[patt]).astype(np.int32)
        ar = np.ascontiguousarray(m.nat_r0[patt]).astype(np.float32)
        R.ref_set_pair_lists(len(ai), P(ai), P(aj), P(ar), len(pri), P(pri), P(prj))
        e = np.zeros(4)
        R.ref_energies(P(e))
        fx[f"{mode}_att"] = patt.astype(np.int32)
        fx[f"{mode}_rep_i"] = pri
        fx[f"{mode}_rep_j"] = prj
        fx[f"{mode}_energy"] = e
    ob = np.zeros(4)
    R.ref_observables(P(ob))
    # output files and the progress line (the absolute-mode lists are the
    # current ones)
    R.ref_set_pos(P(x))
    outs = [os.path.join(HERE, f"m128_out.{k}") for k in ("traj", "traj_unc", "coord", "unccoord", "vel")]
    for o in outs:
        if os.path.exists(o):
            os.remove(o)
    R.ref_write_outputs(*[o.encode() for o in outs])
    line = ctypes.create_string_buffer(1024)
    R.ref_update_line(ctypes.c_double(1000.0), line, 1024)
    with open(os.path.join(HERE, "m128_update.txt"), "w") as f:
        f.write(line.value.decode() + "\n")
    np.savez_compressed(os.path.join(HERE, "m128_energy.npz"), x=x, v=v, observables=ob,
                        coeff_att_11=np.float32(0.7), **fx)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
