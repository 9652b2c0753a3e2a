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
                               observables (sop.cu:528-611) on them.  The
                               factor-mode lists are the reference's own: its
                               host filters update_neighbor_list and
                               update_pair_list (sop.cu:1351-1448, 1707-1823).
                               The reference has no absolute cut-off mode; the
                               absolute-mode (32 / 16 A) lists come from the
                               oracle and serve only as a larger input to the
                               reference's energy routines
  m128_out.{traj,traj_unc,coord,unccoord,vel}
                               the reference's output writers (io.cpp:261-381)
                               on that state (wrapped = unwrapped coordinates)
  m128_update.txt              its progress line for step 1000 (sop.cu:256-259)
  ref_gasdev.npz               the first 3,000 deviates of the reference's host
                               Gaussian generator (random_generator.cpp:83-143)
                               after `set run 7` and `set run 0`
  ref_lists.npz                the reference's host-filter neighbour and pair
                               lists (factor mode, sop.cu:1351-1448, 1707-1823)
                               for every structure of cases.py: sorted pair
                               keys for the 128-bead cases, SHA-256 digests of
                               the sorted keys and the counts for the
                               4,000-bead ones
  ref_rgsq.npz                 the reference's Rg^2 (calculate_observables,
                               sop.cu:563-580, float accumulation) on every
                               structure of cases.py

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

sys.path.insert(0, HERE)
import cases  # noqa: E402


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
    # factor mode: the reference's own host filters on these coordinates
    R.ref_set_state(P(x), P(v))
    R.ref_host_lists_prepare()
    ref = O.ref_lists(R)
    nat_key = {(int(a), int(b)): k for k, (a, b) in enumerate(zip(m.nat_i, m.nat_j))}
    ref_patt = np.array([nat_key[(min(a, b), max(a, b))] for a, b in
                         zip(*ref["pl_att"][:2])], np.int32)
    for mode, (nlf, nla, plf, pla) in {"factor": (3.2, 0.0, 2.5, 0.0),
                                       "absolute": (0.0, 32.0, 0.0, 16.0)}.items():
        if mode == "factor":
            patt = ref_patt
            pri, prj = ref["pl_rep"][0], ref["pl_rep"][1]
        else:
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
    reference_case_lists(R)
    dev = {}
    for run in (7, 0):
        g = np.zeros(3000)
        R.ref_gasdev(run, 3000, P(g))
        dev[f"run{run}"] = g
    np.savez_compressed(os.path.join(HERE, "ref_gasdev.npz"), **dev)
    print("golden fixtures written to", HERE)


def reference_case_lists(R):
    """ref_lists.npz and ref_rgsq.npz: the reference's host filters and its
    Rg^2 on every case."""
    import tempfile
    out, rg = {}, {}
    with tempfile.TemporaryDirectory() as d:
        for name in cases.CASES:
            mol, x, _, boxl = cases.build(name)
            O.ref_load_molecule(R, mol, x, boxl, os.path.join(d, name))
            x32 = np.ascontiguousarray(x, np.float32)
            R.ref_set_state(P(x32), None)
            ob = np.zeros(4)
            R.ref_observables(P(ob))
            rg[name] = np.float64(ob[1])
            R.ref_host_lists_prepare()
            lists = O.ref_lists(R)
            for which, (i, j, _) in lists.items():
                keys = cases.pair_keys(mol.n, i, j)
                out[f"{name}.{which}.count"] = np.int64(len(keys))
                if name in cases.SMALL:
                    out[f"{name}.{which}"] = keys
                else:
                    out[f"{name}.{which}.sha256"] = np.array(cases.digest(keys))
            print(name, {k: len(v[0]) for k, v in lists.items()})
    np.savez_compressed(os.path.join(HERE, "ref_lists.npz"), **out)
    np.savez_compressed(os.path.join(HERE, "ref_rgsq.npz"), **rg)


if __name__ == "__main__":
    main()
