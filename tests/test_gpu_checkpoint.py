"""Exact checkpoints (sop_checkpoint / sop_restore, sop_serve_checkpoint /
sop_serve_resume), through the C ABI: a run continued from a checkpoint in a
fresh context is bit-identical to the run that was never interrupted --
coordinates, velocities, forces and energies -- at any step for plain and
batched contexts, and between rounds for served jobs."""
import numpy as np
import pytest

from sop_gb300 import engine, system

pytestmark = pytest.mark.gpu

_MOLS = {}


def mol_of(n, seed):
    if (n, seed) not in _MOLS:
        _MOLS[(n, seed)] = system.generate(n, seed)
    return _MOLS[(n, seed)]


def state(e, m=0):
    d = e.download(m)
    return d["unc_pos"], d["vel"], d["force"], e.energy(m)


def same(a, b):
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("at", [137, 149, 150])
def test_plain_continues_bit_identically(at):
    mol = mol_of(900, 3)
    p = engine.baseline_params()
    with engine.plain(mol, mol.xyz, p, T=0.65, traj=4) as e:
        e.step(at)
        blob = e.checkpoint(0)
        e.step(300 - at)
        ref = state(e)
        assert e.status(0) == (0, 300)
    with engine.plain(mol, mol.xyz, p, T=0.65, traj=4) as e:
        e.restore(0, blob)
        assert e.status(0) == (0, at)
        e.step(300 - at)
        assert e.status(0) == (0, 300)
        same(state(e), ref)


def test_batched_continues_bit_identically():
    mols = [mol_of(300, 5), mol_of(1200, 6), mol_of(80, 7)]
    p = engine.baseline_params()

    def build():
        e = engine.Engine(p)
        for k, m in enumerate(mols):
            e.add(m, m.xyz, T=0.55 + 0.05 * k, traj=10 + k)
        e.commit()
        return e

    e = build()
    e.step(73)
    blobs = [e.checkpoint(k) for k in range(len(mols))]
    e.step(127)
    ref = [state(e, k) for k in range(len(mols))]
    e.close()
    e = build()
    for k, b in enumerate(blobs):
        e.restore(k, b)
    e.step(127)
    for k in range(len(mols)):
        same(state(e, k), ref[k])
    e.close()


def test_restore_rejects_foreign_and_misaligned_checkpoints():
    p = engine.baseline_params()
    a, b = mol_of(300, 5), mol_of(80, 7)
    with engine.plain(a, a.xyz, p) as e:
        e.step(20)
        blob_a20 = e.checkpoint(0)
        e.step(10)
        blob_a30 = e.checkpoint(0)
    with engine.plain(b, b.xyz, p) as e:
        with pytest.raises(engine.SopError):
            e.restore(0, blob_a20)          # another molecule
        with pytest.raises(engine.SopError):
            e.restore(0, b"not a checkpoint")
    e = engine.Engine(p)
    e.add(a, a.xyz)
    e.add(a, a.xyz, traj=1)
    e.commit()
    e.restore(0, blob_a20)
    with pytest.raises(engine.SopError):
        e.restore(1, blob_a30)              # one clock per context
    e.close()


def test_served_job_resumes_bit_identically():
    p = engine.baseline_params(boxl=12000.0)
    m1, m2 = mol_of(700, 32), mol_of(250, 33)
    with engine.Server(p, 64 << 20, 4000) as srv:
        j1 = srv.submit(m1, m1.xyz, 400, 0.6, traj=1)
        j2 = srv.submit(m2, m2.extended_xyz(), 260, 0.7, traj=2)
        srv.advance(3)                      # admission round, then two more: step 100
        blob = srv.checkpoint(j1)
        srv.run_until_idle()
        ref = srv.result(j1)
        other = srv.result(j2)
    ok = lambda st: st & (engine.MOL_FENE_RANGE | engine.MOL_NONFINITE) == 0  # noqa: E731
    assert ref["steps"] == 400 and ok(ref["status"]) and ok(other["status"])
    with engine.Server(p, 64 << 20, 4000) as srv:
        # the resumed job shares the context with a different job
        srv.submit(m2, m2.xyz, 180, 0.5, traj=3)
        j = srv.resume(m1, blob, 400, 0.6, traj=1)
        srv.run_until_idle()
        got = srv.result(j)
    assert got["steps"] == 400 and got["status"] == ref["status"]
    for k in ("unc_pos", "vel", "energy"):
        np.testing.assert_array_equal(got[k], ref[k])


def test_restore_into_a_context_built_from_other_coordinates():
    """A checkpoint of a fully extended chain (15,200 A, past a quarter of its
    40,000 A box, where the minimum image matters) restored into a context
    committed from the compact native structure: the continuation is still
    bit-identical (the restore refreshes the cell order and grid flags)."""
    mol = mol_of(4000, 1)
    p = engine.baseline_params(boxl=40000.0)
    with engine.plain(mol, mol.extended_xyz(), p, T=0.6, traj=3) as e:
        e.step(60)
        blob = e.checkpoint(0)
        e.step(90)
        ref = state(e)
    with engine.plain(mol, mol.xyz, p, T=0.6, traj=3) as e:
        e.restore(0, blob)
        e.step(90)
        same(state(e), ref)
