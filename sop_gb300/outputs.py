"""The reference's output files, written from this engine's state so a run
leaves the files a run of the reference leaves.

  record_traj     trajectory frames, "%f %f %f" per bead, appended
                  (io.cpp:261-282)
  save_coords     coordinate files, "%d %f %f %f" per bead, 1-based, rewritten
                  (io.cpp:284-305); save_unccoords the unwrapped file alone
                  (io.cpp:307-320)
  save_vels       velocity file, "%d %f %f %f" per bead, appended
                  (io.cpp:365-381)
  load_coords     the reader of coordinate files (io.cpp:322-363)
  update_line     one line of the progress file written every nup steps
                  (sop.cu:256-259)

The reference keeps these quantities in FP32 and prints them with %f (the
float promoted to double); the writers round to FP32 first, so the text is
the same character for character.
"""
from __future__ import annotations

import numpy as np


def _f32(a) -> np.ndarray:
    return np.asarray(a, np.float32).reshape(-1, 3)


def _lines3(a: np.ndarray, numbered: bool) -> str:
    out = []
    for k, (x, y, z) in enumerate(a.tolist()):
        if numbered:
            out.append("%d %f %f %f\n" % (k + 1, x, y, z))
        else:
            out.append("%f %f %f\n" % (x, y, z))
    return "".join(out)


def record_traj(path: str, path_unc: str, pos, unc_pos) -> None:
    """Appends one frame of wrapped and unwrapped coordinates."""
    with open(path, "a") as f:
        f.write(_lines3(_f32(pos), False))
    with open(path_unc, "a") as f:
        f.write(_lines3(_f32(unc_pos), False))


def save_coords(path: str, path_unc: str, pos, unc_pos) -> None:
    """Rewrites the wrapped and unwrapped coordinate files."""
    with open(path, "w") as f:
        f.write(_lines3(_f32(pos), True))
    with open(path_unc, "w") as f:
        f.write(_lines3(_f32(unc_pos), True))


def save_unccoords(path: str, unc_pos) -> None:
    with open(path, "w") as f:
        f.write(_lines3(_f32(unc_pos), True))


def save_vels(path: str, vel) -> None:
    """Appends one velocity frame."""
    with open(path, "a") as f:
        f.write(_lines3(_f32(vel), True))


def load_coords(path: str, path_unc: str, nbead: int) -> tuple[np.ndarray, np.ndarray]:
    """(pos, unc_pos) of the first nbead lines of two coordinate files."""
    def read(p):
        out = np.zeros((nbead, 3), np.float32)
        with open(p) as f:
            for i in range(nbead):
                tok = f.readline().split()
                out[i] = [float(t) for t in tok[1:4]]
        return out
    return read(path), read(path_unc)


def update_line(istep: float, T: float, kinT: float, energy, Q: float, contct_nat: int,
                rgsq: float) -> str:
    """The progress line: step, T, kinT, e_bnd, e_ang_ss, e_vdw_rr_att,
    e_vdw_rr_rep, e_vdw_rr, rna_etot, Q, contct_nat, rgsq.  energy is the
    engine's five terms (bonds, angles, attraction, repulsion, total); the
    sums are re-formed in FP32 as the reference forms them (energy.cu:75,
    energy.cu:440)."""
    f = np.float32
    e_bnd, e_ang, e_att, e_rep = (f(v) for v in list(energy)[:4])
    e_vdw = f(e_att + e_rep)
    etot = f(f(e_bnd + e_ang) + e_vdw)
    vals = (float(istep), float(f(T)), float(f(kinT)), float(e_bnd), float(e_ang), float(e_att),
            float(e_rep), float(e_vdw), float(etot), float(f(Q)), int(contct_nat), float(f(rgsq)))
    return "%.0f %f %f %f %f %f %f %f %f %f %d %f" % vals
