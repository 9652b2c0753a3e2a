"""GPU parity of the plain path against the oracle (through the C ABI).

Lists: bit-exact as sets (the engine's FP32 predicate is the reference's host
filter).  Forces: max relative error <= 1e-5 against FP64 on the same FP32
coordinates and lists (per-bead |dF| / |F|, |F| floored at 1e-3 of the RMS
bead force).  Single steps: identical injected noise.
"""
import numpy as np
import pytest

from helpers import att_sel, force_error, force_error_report, oracle_lists, pairset
from oracle import pyoracle as O
from sop_gb300 import engine, system

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5

_MOLS = {}


def mol_of(n, seed, eps_range=None):
    key = (n, seed, eps_range)
    if key not in _MOLS:
        _MOLS[key] = system.generate(n, seed, eps_range)
    return _MOLS[key]


def perturbed(mol, sigma, seed=0):
    rng = np.random.default_rng(seed)
    return (mol.xyz + rng.normal(0.0, sigma, mol.xyz.shape)).astype(np.float32)


def params(mode, **kw):
    if mode == "factor":
        return engine.default_params(h=0.05, zeta=0.05, **kw)
    return engine.baseline_params(**kw)


def gpu_lists(e, mol):
    ai, aj, ar = e.list_pairs(0, 0)
    ri, rj, _ = e.list_pairs(0, 1)
    pai, paj, par = e.list_pairs(0, 2)
    pri, prj, _ = e.list_pairs(0, 3)
    return (ai, aj, ar), (ri, rj), (pai, paj, par), (pri, prj)


@pytest.mark.parametrize("n,seed", [(128, 0), (4000, 1)])
@pytest.mark.parametrize("mode", ["factor", "absolute"])
@pytest.mark.parametrize("sigma", [0.0, 0.4])
def test_lists_bit_exact(n, seed, mode, sigma):
    mol = mol_of(n, seed)
    x = perturbed(mol, sigma, seed + 7)
    p = params(mode)
    with engine.plain(mol, x, p) as e:
        (ai, aj, ar), (ri, rj), (pai, paj, par), (pri, prj) = gpu_lists(e, mol)
    nl_att, (nri, nrj), pl_att, (opi, opj) = oracle_lists(mol, x, p)
    assert pairset(ai, aj) == pairset(mol.nat_i[nl_att], mol.nat_j[nl_att])
    assert pairset(ri, rj) == pairset(nri, nrj)
    assert pairset(pai, paj) == pairset(mol.nat_i[pl_att], mol.nat_j[pl_att])
    assert pairset(pri, prj) == pairset(opi, opj)
    # the attractive entries carry their native distance unchanged
    sel = att_sel(mol, pai, paj)
    np.testing.assert_array_equal(par, mol.nat_r0[sel])
    assert len(pri) > 0


@pytest.mark.parametrize("n,seed", [(128, 0), (4000, 1)])
@pytest.mark.parametrize("mode", ["factor", "absolute"])
@pytest.mark.parametrize("sigma", [0.0, 0.25])
def test_forces_vs_fp64(n, seed, mode, sigma):
    # sigma (A per axis) keeps every bond well inside the FENE range |r - r0| < R0;
    # a larger perturbation breaks bonds, where the force is undefined and the
    # engine stops the molecule (tested in test_fene_range_is_flagged).
    mol = mol_of(n, seed)
    x = perturbed(mol, sigma, seed + 11)
    with engine.plain(mol, x, params(mode)) as e:
        e.set_noise(np.zeros((mol.n, 3), np.float32))
        e.force_eval()
        assert e.status(0)[0] == 0
        f = e.download()["force"]
        pai, paj, _ = e.list_pairs(0, 2)
        pri, prj, _ = e.list_pairs(0, 3)
    fo, _ = O.forces_f64(mol, x, att_sel(mol, pai, paj), pri, prj)
    err = force_error(f, fo)
    rep = force_error_report(f, fo)
    print(n, mode, sigma, rep)
    assert err <= FORCE_TOL, (err, rep)


def test_forces_per_contact_epsilon():
    mol = mol_of(4000, 2, (0.7, 1.3))
    x = perturbed(mol, 0.3, 5)
    with engine.plain(mol, x, params("absolute")) as e:
        e.set_noise(np.zeros((mol.n, 3), np.float32))
        e.force_eval()
        f = e.download()["force"]
        pai, paj, _ = e.list_pairs(0, 2)
        pri, prj, _ = e.list_pairs(0, 3)
    fo, _ = O.forces_f64(mol, x, att_sel(mol, pai, paj), pri, prj)
    assert force_error(f, fo) <= FORCE_TOL


def test_rep6_forces_and_energy_vs_fp64():
    """The pure 6-power repulsion (rep6 = 1; the reference's form is 12+6):
    forces within 1e-5 and energies within 2e-5 of FP64."""
    mol = mol_of(4000, 1)
    x = perturbed(mol, 0.25, 13)
    with engine.plain(mol, x, params("absolute", rep6=1)) as e:
        e.set_noise(np.zeros((mol.n, 3), np.float32))
        e.force_eval()
        assert e.status(0)[0] == 0
        f = e.download()["force"]
        t = e.energy()
        pai, paj, _ = e.list_pairs(0, 2)
        pri, prj, _ = e.list_pairs(0, 3)
    fo, eo = O.forces_f64(mol, x, att_sel(mol, pai, paj), pri, prj, params={"rep6": 1})
    assert force_error(f, fo) <= FORCE_TOL
    np.testing.assert_allclose(t[:4], eo, rtol=2e-5, atol=1e-6)
    f12, _ = O.forces_f64(mol, x, att_sel(mol, pai, paj), pri, prj)
    assert force_error(f, f12) > 1e-3   # the flag changes the physics


def test_tiny_molecules_beside_a_large_one():
    """Chains of 3 to 8 beads (no native contacts below 4 beads, no
    repulsive pairs below 4, chain ends everywhere) batched with a 4000-bead
    molecule: lists bit-exact, forces within 1e-5 of FP64, and 50 steps
    without an error flag."""
    mols = [mol_of(n, 30 + n) for n in (3, 4, 5, 6, 8)] + [mol_of(4000, 1)]
    p = params("absolute")
    e = engine.Engine(p)
    xs = []
    for k, m in enumerate(mols):
        x = perturbed(m, 0.1, 40 + k)
        xs.append(x)
        e.add(m, x, T=0.6, traj=k)
    e.commit()
    e.set_noise(np.zeros((sum(m.n for m in mols), 3), np.float32))
    e.force_eval()
    for k, (m, x) in enumerate(zip(mols, xs)):
        ai, aj, _ = e.list_pairs(k, 0)
        ri, rj, _ = e.list_pairs(k, 1)
        pai, paj, _ = e.list_pairs(k, 2)
        pri, prj, _ = e.list_pairs(k, 3)
        nl_att, (nri, nrj), pl_att, (opi, opj) = oracle_lists(m, x, p)
        assert pairset(ai, aj) == pairset(m.nat_i[nl_att], m.nat_j[nl_att])
        assert pairset(ri, rj) == pairset(nri, nrj)
        assert pairset(pai, paj) == pairset(m.nat_i[pl_att], m.nat_j[pl_att])
        assert pairset(pri, prj) == pairset(opi, opj)
        if m.n < 4:
            assert len(ri) == 0 and len(m.nat_i) == 0
        fo, _ = O.forces_f64(m, x, att_sel(m, pai, paj), pri, prj)
        assert force_error(e.download(k)["force"], fo) <= FORCE_TOL, m.n
    e.set_noise(None)
    e.step(50)
    for k in range(len(mols)):
        st, n = e.status(k)
        assert st == 0 and n == 50
    e.close()


def test_commit_without_molecules_is_refused():
    e = engine.Engine(params("absolute"))
    with pytest.raises(engine.SopError) as ei:
        e.commit()
    assert ei.value.code == 1   # SOP_ERR_ARG
    e.close()


@pytest.mark.parametrize("mode", ["factor", "absolute"])
def test_energy_vs_fp64(mode):
    mol = mol_of(4000, 1)
    x = perturbed(mol, 0.3, 3)
    with engine.plain(mol, x, params(mode)) as e:
        t = e.energy()
        pai, paj, _ = e.list_pairs(0, 2)
        pri, prj, _ = e.list_pairs(0, 3)
    _, eo = O.forces_f64(mol, x, att_sel(mol, pai, paj), pri, prj)
    np.testing.assert_allclose(t[:4], eo, rtol=2e-5, atol=1e-6)
    np.testing.assert_allclose(t[4], eo.sum(), rtol=2e-5)


@pytest.mark.parametrize("mode", ["factor", "absolute"])
def test_energy_and_observables_vs_reference_golden(mode):
    """GPU energies and observables against the reference's own host routines
    (fixtures of tests/golden/make_golden.py), with the reference's energy
    coefficient for native pairs (coeff_att[1][1] = 0.7, global.cpp:51-55)."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "m128_energy.npz"))
    mol = mol_of(128, 0)
    eps_e = np.full(len(mol.nat_i), float(g["coeff_att_11"]), np.float32)
    with engine.plain(mol, g["x"], params(mode), vel=g["v"], eps_energy=eps_e) as e:
        t = e.energy()
        ob = e.observables()
    np.testing.assert_allclose(t[:4], g[f"{mode}_energy"], rtol=2e-5, atol=1e-5)
    q, rg, kin, cnt = g["observables"]
    assert ob["contct_nat"] == int(cnt)
    assert ob["rgsq"] == pytest.approx(rg, rel=2e-6)
    assert ob["kinT"] == pytest.approx(kin, rel=2e-6)


def test_observables_vs_fp64():
    mol = mol_of(4000, 1)
    x = perturbed(mol, 1.0, 4)
    rng = np.random.default_rng(9)
    v = rng.normal(0, 0.8, x.shape).astype(np.float32)
    with engine.plain(mol, x, params("absolute"), vel=v) as e:
        ob = e.observables()
    oo = O.observables(mol, x, v)
    assert ob["contct_nat"] == oo["contct_nat"]
    assert ob["Q"] == pytest.approx(oo["Q"], abs=1e-12)
    assert ob["rgsq"] == pytest.approx(oo["rgsq"], rel=1e-9)
    assert ob["kinT"] == pytest.approx(oo["kinT"], rel=1e-9)


def test_philox_noise_matches_oracle():
    mol = mol_of(4000, 1)
    T, traj = 0.7, 3
    p = params("absolute", seed=0x1234_5678_9ABC)
    with engine.plain(mol, mol.xyz, p, T=T, traj=traj) as e:
        e.set_noise(np.zeros((mol.n, 3), np.float32))
        e.force_eval()
        f0 = e.download()["force"].astype(np.float64)
        e.set_noise(None)
        e.force_eval()
        f1 = e.download()["force"].astype(np.float64)
    sig = O.langevin_consts(0.05, 0.05, T)[4]
    z = (f1 - f0) / sig
    zo = O.noise_normals(mol.n, 0, traj, 0x1234_5678_9ABC)
    np.testing.assert_allclose(z, zo, atol=2e-5)
    assert abs(z.mean()) < 0.05 and abs(z.std() - 1.0) < 0.05


def _oracle_steps(mol, x0, v0, z, T, h, zeta, nsteps, p, boxl=500.0):
    """FP64 oracle trajectory with the engine's cadence and the same injected
    normals z every step; lists from the FP32 positions as the engine keeps them."""
    c = O.langevin_consts(h, zeta, T)
    x = x0.astype(np.float64)
    pos = x.copy()
    v = v0.astype(np.float64)
    xf = x0.astype(np.float32)
    nl = oracle_lists(mol, xf, p, boxl)
    nl_att, (nri, nrj) = nl[0], nl[1]
    pl_att, (pri, prj) = nl[2], nl[3]
    f, _ = O.forces_f64(mol, xf, pl_att, pri, prj)
    f += c[4] * z
    incr = np.zeros_like(x)
    for n in range(1, nsteps + 1):
        if n % p.nnlup == 0:
            nl_att = O.filter_att(mol, xf, None, p.nl_att_fac, p.nl_att_abs, boxl)
            nri, nrj = O.nl_rep(mol, xf, p.nl_rep_fac, p.nl_rep_abs, boxl)
        if n % p.nnlup == 0 or p.nplup <= 1 or n % p.nplup == 0:
            pl_att = O.filter_att(mol, xf, nl_att, p.pl_att_fac, p.pl_att_abs, boxl)
            pri, prj = O.filter_rep(mol, xf, nri, nrj, p.pl_rep_fac, p.pl_rep_abs, boxl)
        incr = c[0] * v + c[1] * f
        x = x + incr
        pos = pos + incr
        pos -= boxl * np.rint(pos / boxl)
        xf = x.astype(np.float32)
        f, _ = O.forces_f64(mol, xf, pl_att, pri, prj)
        f += c[4] * z
        v = c[2] * incr + c[3] * f
    return x, v, f


@pytest.mark.parametrize("mode,nsteps", [("factor", 1), ("absolute", 1), ("factor", 12)])
def test_steps_with_injected_noise(mode, nsteps):
    mol = mol_of(128, 0)
    x0 = perturbed(mol, 0.2, 1)
    rng = np.random.default_rng(2)
    v0 = rng.normal(0, 0.5, x0.shape).astype(np.float32)
    z = rng.normal(0, 1, x0.shape).astype(np.float32)
    T = 0.6
    p = params(mode, nnlup=5, nplup=1 if mode == "factor" else 2)
    with engine.plain(mol, x0, p, T=T, vel=v0) as e:
        e.set_noise(z)
        e.force_eval()
        e.step(nsteps)
        st = e.download()
        assert e.status(0) == (0, nsteps)
    x, v, f = _oracle_steps(mol, x0, v0, z.astype(np.float64), T, 0.05, 0.05, nsteps, p)
    assert force_error(st["force"], f) <= (FORCE_TOL if nsteps == 1 else 1e-4)
    np.testing.assert_allclose(st["unc_pos"], x, atol=5e-5 * nsteps)
    np.testing.assert_allclose(st["vel"], v, atol=2e-4 * nsteps, rtol=1e-4)


def test_deterministic_and_graph_equals_eager():
    mol = mol_of(4000, 1)
    outs = []
    for gs in (10, 10, 4):
        p = engine.baseline_params(graph_steps=gs)
        with engine.plain(mol, mol.xyz, p, T=0.6, traj=1) as e:
            e.step(3)   # eager partial block
            e.step(57)  # graph replays + an eager tail
            outs.append(e.download())
    for k in ("unc_pos", "vel", "force", "pos"):
        np.testing.assert_array_equal(outs[0][k], outs[1][k])
        np.testing.assert_array_equal(outs[0][k], outs[2][k])


def test_state_upload_touches_only_its_molecule():
    """sop_upload_state rebuilds the lists of the molecule it loads and no
    other: a finished molecule keeps the lists of its last step (its energy
    is evaluated on them) and a running one continues bit-identically to a
    run alone, also when the upload's neighbour list overflows the row
    stride and the rows regrow.  The rows are sized at commit for the
    densest synthetic globules, so the overflow comes from the folded
    structure shrunk to half its size (eight times as dense)."""
    a, b, c = mol_of(128, 0), mol_of(4000, 1), mol_of(300, 5)
    p = engine.baseline_params(boxl=40000.0)
    e = engine.Engine(p)
    e.add(a, a.xyz, T=0.6, traj=0, nsteps=20)
    e.add(b, b.extended_xyz(), T=0.6, traj=1)
    e.add(c, c.xyz, T=0.7, traj=2)
    e.commit()
    e.step(30)
    assert e.status(0)[1] == 20 and e.status(1) == (0, 30)
    before = [e.energy(0), *e.list_pairs(0, 1), *e.list_pairs(0, 3), *e.list_pairs(2, 3)]
    bytes0 = e.memory(0)[0]
    dense = (b.xyz - b.xyz.mean(0)) * 0.5 + b.xyz.mean(0)
    e.upload_state(1, dense.astype(np.float32))
    assert e.memory(0)[0] > bytes0    # the rows regrew
    e.upload_state(1, b.xyz)          # the folded structure, in the regrown rows
    after = [e.energy(0), *e.list_pairs(0, 1), *e.list_pairs(0, 3), *e.list_pairs(2, 3)]
    for x, y in zip(after, before):
        np.testing.assert_array_equal(x, y)
    _, (nri, nrj), _, (opi, opj) = oracle_lists(b, b.xyz, p, 40000.0)
    ri, rj, _ = e.list_pairs(1, 1)
    pri, prj, _ = e.list_pairs(1, 3)
    assert pairset(ri, rj) == pairset(nri, nrj)
    assert pairset(pri, prj) == pairset(opi, opj)
    e.step(40)
    mixed = e.download(2)
    e.close()
    with engine.plain(c, c.xyz, p, T=0.7, traj=2) as alone:
        alone.step(70)
        ref = alone.download()
    for k in ("unc_pos", "vel", "force"):
        np.testing.assert_array_equal(mixed[k], ref[k])


def test_rows_regrow_mid_run():
    """A neighbour-list row that outgrows the row stride at a rebuild inside a
    running block of steps: every molecule freezes at the start of that block,
    the rows regrow (keeping every molecule's lists) and the block runs again.
    The trajectory is the one of a context whose rows had room from the
    start, bit for bit.  The start is the folded 4,000-bead structure
    expanded by 1.3 about its centre, moving inwards (v = -0.03 (x - c) per
    unit time): its longest row grows from 289 entries at the start to
    about 360 at step 50 and 540 at step 200, past rows of 320 entries and
    then past the regrown ones."""
    mol = system.generate(4000, 1)
    c = mol.xyz.mean(0)
    x0 = ((mol.xyz - c) * 1.3 + c).astype(np.float32)
    v0 = (-0.03 * (x0 - c)).astype(np.float32)
    with engine.plain(mol, x0, engine.baseline_params(nl_rows=300), T=0.6, traj=3, vel=v0) as e:
        m0 = e.memory(0)[0]
        e.step(300)
        grown = e.memory(0)[0] > m0
        assert e.status(0)[0] == 0
        a = e.download()
    with engine.plain(mol, x0, engine.baseline_params(), T=0.6, traj=3, vel=v0) as e:
        e.step(300)
        b = e.download()
    assert grown
    for k in ("unc_pos", "vel", "force"):
        np.testing.assert_array_equal(a[k], b[k])


@pytest.mark.parametrize("boxl", [40000.0, 500.0])
def test_extended_chain_lists(boxl):
    """Extended start: with a large box the cell grid is a long row; with the
    reference's 500 A box the chain wraps, the minimum image matters and the
    all-pairs scan is used."""
    mol = mol_of(1500, 3)
    x = mol.extended_xyz()
    p = params("absolute", boxl=boxl)
    with engine.plain(mol, x, p) as e:
        _, (ri, rj), _, (pri, prj) = gpu_lists(e, mol)
    _, (nri, nrj), _, (opi, opj) = oracle_lists(mol, x, p, boxl)
    assert pairset(ri, rj) == pairset(nri, nrj)
    assert pairset(pri, prj) == pairset(opi, opj)


def test_lists_of_more_than_a_thousand_molecules():
    """The per-molecule cell bases come from a block-wide scan with 1,024
    threads, one molecule per thread: 1,100 copies of a 1,000-bead molecule
    in one context put molecules 992-1,023 in the block's last warp (whose
    prefix a scan that kept its total in that warp's slot got wrong).  Every
    copy's lists equal the oracle's."""
    mol = mol_of(1000, 5)
    p = engine.baseline_params()
    ncopy = 1100
    with engine.Engine(p) as e:
        for k in range(ncopy):
            e.add(mol, mol.xyz, T=0.6, traj=k)
        e.commit()
        nl_att, (nri, nrj), pl_att, (opi, opj) = oracle_lists(mol, mol.xyz, p)
        want_nl, want_pl = pairset(nri, nrj), pairset(opi, opj)
        for k in (0, 500, 991, 992, 1000, 1023, 1024, 1030, 1060, 1099):
            ri, rj, _ = e.list_pairs(k, 1)
            pri, prj, _ = e.list_pairs(k, 3)
            assert pairset(ri, rj) == want_nl, k
            assert pairset(pri, prj) == want_pl, k


def test_batched_equals_alone():
    """Molecules packed into one context give bit-identical results to the
    same molecules run alone."""
    sizes = [(90, 10), (700, 11), (1500, 12)]
    mols = [mol_of(n, s) for n, s in sizes]
    p = engine.baseline_params()
    alone = []
    for k, m in enumerate(mols):
        with engine.plain(m, m.xyz, p, T=0.5 + 0.1 * k, traj=k) as e:
            e.step(40)
            alone.append(e.download())
    with engine.Engine(p) as e:
        for k, m in enumerate(mols):
            e.add(m, m.xyz, T=0.5 + 0.1 * k, traj=k)
        e.commit()
        e.step(40)
        for k in range(len(mols)):
            d = e.download(k)
            for key in ("unc_pos", "vel", "force"):
                np.testing.assert_array_equal(d[key], alone[k][key])


def test_lanes_per_bead_bit_identical():
    """The force summation order does not depend on the lanes per bead, and
    every form of the step (one kernel; force + finish kernels; the steps
    between two rebuilds in one persistent launch, over the grid or in one
    block) completes a bead with the same code, so trajectories are
    bit-identical for every G and form (both can be tuned freely)."""
    mol = mol_of(4000, 1)
    outs = []
    for g in (2, 4, 8, 16):
        for form in (1, 2, 3, 4):
            p = engine.baseline_params(lanes_per_bead=g, step_split=form)
            with engine.plain(mol, mol.xyz, p, T=0.6, traj=2) as e:
                t = e.tuning()
                assert t["lanes_per_bead"] == g and t["form"] == form
                e.step(30)
                outs.append(e.download())
    for o in outs[1:]:
        for k in ("unc_pos", "vel", "force"):
            np.testing.assert_array_equal(o[k], outs[0][k])


def test_one_block_form_small_context():
    """The one-block form on a context it is meant for (128 beads, every lane
    count): bit-identical to the one-kernel form over 120 steps (list
    rebuilds included), and the tuner may pick it."""
    mol = mol_of(128, 0)
    outs = []
    for g, form in ((16, 1), (2, 4), (4, 4), (8, 4), (16, 4)):
        p = engine.baseline_params(lanes_per_bead=g, step_split=form)
        with engine.plain(mol, mol.xyz, p, T=0.6, traj=4) as e:
            assert e.tuning()["form"] == form
            e.step(120)
            outs.append(e.download())
    for o in outs[1:]:
        for k in ("unc_pos", "vel", "force"):
            np.testing.assert_array_equal(o[k], outs[0][k])
    with engine.plain(mol, mol.xyz, engine.baseline_params(), T=0.6, traj=4) as e:
        assert e.tuning()["form"] in (1, 2, 4)


def test_step_window_bit_identical():
    """Blocks that stage their molecules in shared memory gather the same
    coordinates as blocks that read global memory, in the same order: a
    batched context of molecules from 40 to 1,800 beads (some blocks fit a
    window, some do not; two bead types in one molecule) steps bit-identically
    with no window, small and large windows, every form and several G."""
    mols = [mol_of(n, 30 + k) for k, n in enumerate((40, 300, 1800, 75, 900, 1200, 60))]
    base = mols[3]
    types = np.where(np.arange(base.n) % 3 == 0, 2, 1).astype(np.int32)
    mols[3] = system.Molecule(base.n, base.xyz, base.bond_i, base.bond_j, base.bond_r0,
                              base.ang_i, base.ang_j, base.ang_k, base.ang_r, base.nat_i,
                              base.nat_j, base.nat_r0, base.nat_eps, types=types)
    outs = []
    for win in (-1, 256, 1024, 2048):
        for g, form in ((4, 1), (8, 2), (16, 1), (8, 3)):
            p = engine.baseline_params(lanes_per_bead=g, step_split=form, step_window=win)
            e = engine.Engine(p)
            for k, m in enumerate(mols):
                e.add(m, m.xyz, T=0.6, traj=k)
            e.commit()
            t = e.tuning()
            assert t["window"] == max(win, 0) and t["lanes_per_bead"] == g
            e.step(60)
            outs.append([e.download(k) for k in range(len(mols))])
            e.close()
    for o in outs[1:]:
        for k in range(len(mols)):
            for key in ("unc_pos", "vel", "force"):
                np.testing.assert_array_equal(o[k][key], outs[0][k][key])


def test_size_bucket_tiles_bit_identical():
    """The per-size-bucket tiled step (each molecule in tiles of its bucket's
    lanes and form, one launch) gives the bits of the whole-context step: a
    batched context with molecules in all three buckets, tiled forced on and
    off; the tuner reports a choice for every bucket."""
    mols = [mol_of(n, 60 + k) for k, n in enumerate((70, 150, 330, 520, 900, 1400, 45))]
    outs = []
    for buckets in (1, -1):
        e = engine.Engine(engine.baseline_params(step_buckets=buckets))
        for k, m in enumerate(mols):
            e.add(m, m.xyz, T=0.6, traj=k)
        e.commit()
        t = e.tuning()["buckets"]
        assert t["tiled"] == (buckets == 1)
        if buckets == 1:
            for name, b in t["by_bucket"].items():
                assert b["beads"] > 0 and b["lanes_per_bead"] in (4, 8) and b["form"] in (1, 2)
            assert t["ms_tiled"] > 0 and t["ms_whole"] > 0
        e.step(60)
        outs.append([e.download(k) for k in range(len(mols))])
        e.close()
    for k in range(len(mols)):
        for key in ("unc_pos", "vel", "force"):
            np.testing.assert_array_equal(outs[0][k][key], outs[1][k][key])


def test_persistent_step_barrier_wait_ends():
    """The persistent form's device-wide barrier completes when every block
    arrives, and when an arrival never comes its wait runs out after the
    limit: the kernel returns, the host reads the flag, and the context keeps
    stepping exactly as a context that never saw it."""
    mol = mol_of(4000, 1)
    p = engine.baseline_params(lanes_per_bead=4, step_split=3)
    with engine.plain(mol, mol.xyz, p, T=0.6, traj=3) as e, \
            engine.plain(mol, mol.xyz, p, T=0.6, traj=3) as ref:
        assert e.tuning()["form"] == 3
        e.step(25)
        assert e.check_step_barrier(0, 1.0) is False
        assert e.check_step_barrier(1, 0.2) is True
        assert e.check_step_barrier(0, 1.0) is False
        e.step(25)
        ref.step(50)
        a, b = e.download(), ref.download()
        for key in ("unc_pos", "vel", "force"):
            np.testing.assert_array_equal(a[key], b[key])


def test_autotune_picks_a_candidate():
    mol = mol_of(4000, 1)
    with engine.plain(mol, mol.xyz, engine.baseline_params()) as e:
        t = e.tuning()
    assert t["lanes_per_bead"] in (2, 4, 8, 16) and t["form"] in (1, 2, 3, 4)
    assert all(v > 0 for v in t["ms"].values())


@pytest.mark.parametrize("mode", ["factor", "absolute"])
def test_two_bead_types(mode):
    """Type-2 beads use sigma_rep 7.0 (5.4 across types, energy.cu:9-13) in the
    repulsion and in the list cut-offs."""
    base = mol_of(1500, 4)
    rng = np.random.default_rng(6)
    types = np.where(rng.random(base.n) < 0.3, 2, 1).astype(np.int32)
    mol = system.Molecule(base.n, base.xyz, base.bond_i, base.bond_j, base.bond_r0, base.ang_i,
                          base.ang_j, base.ang_k, base.ang_r, base.nat_i, base.nat_j, base.nat_r0,
                          base.nat_eps, types=types)
    x = perturbed(mol, 0.2, 8)
    p = params(mode)
    with engine.plain(mol, x, p) as e:
        e.set_noise(np.zeros((mol.n, 3), np.float32))
        e.force_eval()
        f = e.download()["force"]
        _, (ri, rj), _, (pri, prj) = gpu_lists(e, mol)
        pai, paj, _ = e.list_pairs(0, 2)
    _, (nri, nrj), _, (opi, opj) = oracle_lists(mol, x, p)
    assert pairset(ri, rj) == pairset(nri, nrj)
    assert pairset(pri, prj) == pairset(opi, opj)
    fo, _ = O.forces_f64(mol, x, att_sel(mol, pai, paj), pri, prj)
    assert force_error(f, fo) <= FORCE_TOL


def test_fene_range_is_flagged():
    """A bond stretched beyond R0 stops the molecule with a status bit instead
    of producing log of a negative number (energy.cu:220 has no guard)."""
    mol = mol_of(128, 0)
    x = mol.xyz.copy()
    x[64:] += np.array([3.0, 0.0, 0.0], np.float32)   # bond 63-64 stretched by ~3 A
    with engine.plain(mol, x, engine.baseline_params()) as e:
        st, n = e.status(0)
        assert st & engine.MOL_FENE_RANGE
        e.step(10)
        assert e.status(0)[1] == 0   # the molecule no longer advances


def test_long_run_stays_folded():
    mol = mol_of(128, 0)
    with engine.plain(mol, mol.xyz, engine.baseline_params(), T=0.6) as e:
        e.step(2000)
        st, n = e.status(0)
        ob = e.observables()
        en = e.energy()
    assert st == 0 and n == 2000
    assert np.all(np.isfinite(en))
    assert ob["Q"] > 0.6
    assert 0.2 < ob["kinT"] < 1.2


def test_overdamped_steps_with_injected_noise():
    """integrator = 1: x += (h / zeta) (F + sigma z) (sop.cu:487-521,
    a5 = h / zeta), against FP64 forces on the same lists; velocities stay 0."""
    mol = mol_of(128, 0)
    x0 = perturbed(mol, 0.2, 1)
    rng = np.random.default_rng(5)
    z = rng.normal(0, 1, x0.shape).astype(np.float32)
    T, h, zeta = 0.6, 0.001, 0.05
    p = engine.baseline_params(integrator=1, h=h, zeta=zeta)
    with engine.plain(mol, x0, p, T=T) as e:
        e.set_noise(z)
        e.force_eval()
        e.step(3)
        st = e.download()
        assert e.status(0) == (0, 3)
        pai, paj, _ = e.list_pairs(0, 2)
        pri, prj, _ = e.list_pairs(0, 3)
        assert e.observables()["kinT"] == 0.0
    a5, sig = h / zeta, np.sqrt(2.0 * T * zeta / h)
    x = x0.astype(np.float64)
    sel = att_sel(mol, pai, paj)
    for _ in range(3):   # no list rebuild within the first 10 steps
        f, _ = O.forces_f64(mol, x.astype(np.float32), sel, pri, prj)
        x = x + a5 * (f + sig * z)
    np.testing.assert_allclose(st["unc_pos"], x, atol=5e-5)
    assert np.all(st["vel"] == 0.0)


def test_download_all_matches_per_molecule_downloads():
    """sop_download_all: every molecule's current coordinates in id order,
    the same as downloading them one by one."""
    mols = [mol_of(128, 0), mol_of(4000, 1), mol_of(300, 5)]
    e = engine.Engine(engine.baseline_params())
    for k, m in enumerate(mols):
        e.add(m, m.xyz, T=0.6, traj=k)
    e.commit()
    e.step(17)
    allx = e.download_all()
    each = np.concatenate([e.download(k)["unc_pos"] for k in range(len(mols))])
    e.close()
    np.testing.assert_array_equal(allx, each)


def test_download_all_async_overlaps_and_matches_blocking_downloads():
    """sop_download_all_async: queued between queued steps, each download
    holds the coordinates of the point in the queue where it was issued (the
    same bits as a blocking download there), with two downloads in flight
    and a third reusing the first one's buffer; bad tickets are refused."""
    torch = pytest.importorskip("torch")
    mols = [mol_of(128, 0), mol_of(4000, 1), mol_of(300, 5)]
    total = sum(m.n for m in mols)

    def make():
        e = engine.Engine(engine.baseline_params())
        for k, m in enumerate(mols):
            e.add(m, m.xyz, T=0.6, traj=k)
        e.commit()
        return e

    ref = make()
    want = []
    for n in (10, 7, 13, 10):
        ref.step(n)
        want.append(ref.download_all().copy())
    ref.close()

    e = make()
    bufs = [torch.empty((total, 3), dtype=torch.float32, pin_memory=True).numpy() for _ in range(4)]
    tickets = []
    for k, n in enumerate((10, 7, 13, 10)):
        e.step_async(n)
        tickets.append(e.download_all_async(bufs[k]))
    got = []
    for t, b in zip(tickets, bufs):
        e.download_wait(t)
        got.append(b.copy())
    e.sync()
    with pytest.raises(engine.SopError) as ei:
        e.download_wait(len(tickets))   # never issued
    assert ei.value.code == 1
    e.close()
    assert tickets == [0, 1, 2, 3]
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, w)


def test_ensemble_contexts_bit_identical():
    """An ensemble split over three contexts on three streams, stepped
    together across neighbour-list rebuilds, gives the bits of one context
    holding every molecule: coordinates (blocking and queued downloads in id
    order), velocities, forces, energies and step counts.  The contexts after
    the first run in its lanes per bead and step form."""
    torch = pytest.importorskip("torch")
    sizes = [(60, 20), (700, 21), (150, 22), (1500, 23), (90, 24), (400, 25), (1200, 26)]
    mols = [mol_of(n, s) for n, s in sizes]
    total = sum(m.n for m in mols)

    def make(parts):
        ens = engine.Ensemble(engine.baseline_params(), parts=parts)
        for k, m in enumerate(mols):
            assert ens.add(m, m.xyz, T=0.5 + 0.05 * k, traj=k) == k
        ens.commit()
        return ens

    one, three = make(1), make(3)
    assert len(one.engines) == 1 and len(three.engines) == 3
    tuned = three.tuning()
    if not tuned[0]["buckets"]["tiled"] and tuned[0]["form"] in (1, 2):
        first = (tuned[0]["lanes_per_bead"], tuned[0]["form"])
        assert all((t["lanes_per_bead"], t["form"]) == first for t in tuned), tuned
    assert three.cuts == engine.split_by_beads([m.n for m in mols], 3)
    buf = torch.empty((total, 3), dtype=torch.float32, pin_memory=True).numpy()
    for ens in (one, three):
        ens.step_async(60)
        ens.step_async(57)
    tickets = three.download_all_async(buf)
    want = one.download_all()
    three.download_wait(tickets)
    np.testing.assert_array_equal(buf, want)
    np.testing.assert_array_equal(three.download_all(), want)
    for k in range(len(mols)):
        a, b = one.download(k), three.download(k)
        for key in ("unc_pos", "vel", "force"):
            np.testing.assert_array_equal(a[key], b[key])
        np.testing.assert_array_equal(one.energy(k), three.energy(k))
        assert one.status(k) == three.status(k) == (0, 117)
    one.close()
    three.close()
