"""Served engine (continuous batching) on the GPU: jobs submitted while others
run, admitted by HBM budget, retired with their results.  Each job's result
is the same as running it alone on the plain path -- bit-identical, because a
job keeps its own step count and list cadence, its lists and cell grid depend
on its own coordinates only, and the force summation order does not depend on
the mix or the lanes per bead."""
import numpy as np
import pytest

from sop_gb300 import engine, system

pytestmark = pytest.mark.gpu

_MOLS = {}


def mol_of(n, seed):
    if (n, seed) not in _MOLS:
        _MOLS[(n, seed)] = system.generate(n, seed)
    return _MOLS[(n, seed)]


JOBS = [  # (n, seed, steps, T, extended start)
    (220, 31, 120, 0.60, False),
    (700, 32, 230, 0.55, True),
    (1500, 33, 160, 0.80, False),
    (90, 34, 300, 0.70, True),
    (1100, 35, 75, 0.65, False),
    (400, 36, 0, 0.50, False),
]


def start_xyz(m, ext):
    return m.extended_xyz() if ext else m.xyz


def alone(n, seed, steps, T, ext, traj, p):
    m = mol_of(n, seed)
    with engine.plain(m, start_xyz(m, ext), p, T=T, traj=traj, nsteps=steps) as e:
        e.step(steps)
        d = e.download()
        return d["unc_pos"], d["vel"], e.energy(), e.status(0)


def params():
    # a box that holds the extended chains without self-images
    return engine.baseline_params(boxl=12000.0)


def test_mix_equals_alone_with_queueing_and_slot_reuse():
    p = params()
    # a budget that holds only part of the stream at once: jobs queue and
    # later ones reuse the slots of earlier ones
    with engine.Server(p, budget_bytes=12 << 20, max_job_beads=1500) as srv:
        cap = srv.stats()["bead_capacity"]
        assert cap < sum(j[0] for j in JOBS)
        ids = [srv.submit(mol_of(n, s), start_xyz(mol_of(n, s), ext), nsteps=st, T=T, traj=100 + k)
               for k, (n, s, st, T, ext) in enumerate(JOBS)]
        seen_queue = False
        for _ in range(200):
            s = srv.stats()
            seen_queue |= s["queued"] > 0 and s["active"] > 0
            if s["queued"] == 0 and s["active"] == 0:
                break
            srv.advance(1)
        assert seen_queue
        done = srv.finished()
        assert sorted(done) == sorted(ids)
        for k, (n, s, st, T, ext) in enumerate(JOBS):
            r = srv.result(ids[k])
            unc, vel, en, (status, steps) = alone(n, s, st, T, ext, 100 + k, p)
            assert r["steps"] == st == steps
            assert r["status"] == engine.MOL_DONE
            assert r["latency_s"] > 0
            np.testing.assert_array_equal(r["unc_pos"], unc)
            np.testing.assert_array_equal(r["vel"], vel)
            np.testing.assert_allclose(r["energy"], en, rtol=0, atol=0)


def test_poisoned_job_is_retired_and_others_continue():
    p = params()
    with engine.Server(p, budget_bytes=256 << 20, max_job_beads=1500) as srv:
        good = [srv.submit(mol_of(n, s), mol_of(n, s).xyz, nsteps=st, T=T, traj=200 + k)
                for k, (n, s, st, T, _) in enumerate(JOBS[:3])]
        bad_m = mol_of(300, 40)
        x = bad_m.xyz.copy()
        x[150:] += np.array([3.0, 0.0, 0.0], np.float32)  # one bond stretched beyond R0
        bad = srv.submit(bad_m, x, nsteps=200, T=0.6, traj=299)
        srv.run_until_idle()
        rb = srv.result(bad)
        assert rb["status"] & engine.MOL_FENE_RANGE
        assert rb["steps"] == 0
        for k, (n, s, st, T, _) in enumerate(JOBS[:3]):
            r = srv.result(good[k])
            unc, vel, _, _ = alone(n, s, st, T, False, 200 + k, p)
            assert r["status"] == engine.MOL_DONE
            np.testing.assert_array_equal(r["unc_pos"], unc)


def test_submit_rejects_oversized_and_stepless_jobs():
    p = params()
    with engine.Server(p, budget_bytes=64 << 20, max_job_beads=500) as srv:
        with pytest.raises(engine.SopError):
            srv.submit(mol_of(700, 32), nsteps=10)
        with pytest.raises(engine.SopError):
            srv.submit(mol_of(220, 31), nsteps=-1)


def test_more_than_a_thousand_jobs_at_once():
    """1,100 jobs resident at once: the molecule slots run past the last warp
    of the 1,024-thread scan of per-molecule cell bases (slots 992-1,023),
    and jobs there must still equal their runs alone."""
    p = params()
    m = mol_of(150, 41)
    njob = 1100
    with engine.Server(p, budget_bytes=2 << 30, max_job_beads=1500) as srv:
        ids = [srv.submit(m, m.xyz, nsteps=60, T=0.6, traj=1000 + k) for k in range(njob)]
        srv.advance(1)
        assert srv.stats()["active"] == njob
        srv.run_until_idle()
        for k in (0, 991, 992, 1000, 1023, 1024, 1099):
            r = srv.result(ids[k])
            unc, vel, _, _ = alone(150, 41, 60, 0.6, False, 1000 + k, p)
            assert r["status"] == engine.MOL_DONE, k
            np.testing.assert_array_equal(r["unc_pos"], unc)
            np.testing.assert_array_equal(r["vel"], vel)
