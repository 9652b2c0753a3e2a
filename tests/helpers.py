"""Shared test helpers: GPU list downloads mapped onto the oracle's inputs,
and the force-error metric."""
import numpy as np

from oracle import pyoracle as O


def native_index(mol):
    return {(int(a), int(b)): k for k, (a, b) in enumerate(zip(mol.nat_i, mol.nat_j))}


def att_sel(mol, ai, aj):
    key = native_index(mol)
    return np.array([key[(int(a), int(b))] for a, b in zip(ai, aj)], np.int64)


def pairset(i, j):
    return set(zip(np.asarray(i).tolist(), np.asarray(j).tolist()))


def force_error(f, fo):
    """Max over beads of |F_gpu - F_64| / |F_64|, with |F_64| floored at 1e-3 of
    the RMS bead force (beads whose net force nearly cancels)."""
    f = np.asarray(f, np.float64)
    fo = np.asarray(fo, np.float64)
    mag = np.linalg.norm(fo, axis=1)
    floor = 1e-3 * np.sqrt((mag ** 2).mean())
    return float((np.linalg.norm(f - fo, axis=1) / np.maximum(mag, floor)).max())


def force_error_report(f, fo):
    """The floored metric of force_error beside what the floor hides: the
    unfloored max relative error, how many beads sit below the floor, and the
    largest absolute error as a fraction of the RMS bead force."""
    f = np.asarray(f, np.float64)
    fo = np.asarray(fo, np.float64)
    mag = np.linalg.norm(fo, axis=1)
    rms = np.sqrt((mag ** 2).mean())
    floor = 1e-3 * rms
    d = np.linalg.norm(f - fo, axis=1)
    return {"floored": float((d / np.maximum(mag, floor)).max()),
            "unfloored": float((d / np.maximum(mag, 1e-300)).max()),
            "beads_below_floor": int((mag < floor).sum()), "beads": int(len(mag)),
            "abs_max_over_rms": float(d.max() / rms)}


def oracle_lists(mol, x, p, boxl=500.0):
    """Oracle NL and PL (att as native indices, rep as (i, j)) for engine params p."""
    nl_att = O.filter_att(mol, x, None, p.nl_att_fac, p.nl_att_abs, boxl)
    nri, nrj = O.nl_rep(mol, x, p.nl_rep_fac, p.nl_rep_abs, boxl)
    pl_att = O.filter_att(mol, x, nl_att, p.pl_att_fac, p.pl_att_abs, boxl)
    pri, prj = O.filter_rep(mol, x, nri, nrj, p.pl_rep_fac, p.pl_rep_abs, boxl)
    return nl_att, (nri, nrj), pl_att, (pri, prj)
