"""CPU-side checks: the C-ABI library loads and exports every declared entry
point, the generator meets the workload specification, Philox matches its
published known-answer vectors, and the oracle's list filters are consistent."""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import pyoracle as O
from sop_gb300 import engine, system

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "sop_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(sop_[a-z_0-9]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(engine.lib_path())
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s


def test_binding_covers_every_declared_symbol():
    engine.lib()  # binds argtypes for each entry point; raises on a missing one
    src = open(os.path.join(ROOT, "sop_gb300", "engine.py")).read()
    for s in declared_symbols():
        assert f'"{s}"' in src, s


def test_params_default_matches_reference():
    p = engine.default_params()
    assert (p.k_bnd, p.R0, p.eps_ss, p.sigma_ss, p.eps_rep, p.boxl) == (20.0, 2.0, 1.0, 3.5, 1.0, 500.0)
    assert (p.h, p.zeta, p.nnlup, p.nplup) == (2.5e-3, 5.0e-2, 50, 1)
    assert (p.nl_att_fac, p.nl_rep_fac, p.pl_att_fac, p.pl_rep_fac) == (3.2, 3.2, 2.5, 2.5)


@pytest.mark.parametrize("field,value", [("lanes_per_bead", 3), ("lanes_per_bead", 32),
                                         ("step_split", 5), ("h", 0.0), ("boxl", -1.0)])
def test_context_refuses_invalid_parameters(field, value):
    """Parameters are checked before any device is touched: an invalid one is
    SOP_ERR_ARG with a message, and no context is made."""
    p = engine.default_params()
    setattr(p, field, value)
    h = ctypes.c_void_p()
    rc = engine.lib().sop_ctx_create(ctypes.byref(p), ctypes.byref(h))
    assert rc == 1 and not h.value  # SOP_ERR_ARG
    assert b"invalid parameters" in engine.lib().sop_last_error(None)


@pytest.mark.parametrize("n,seed", [(128, 0), (4000, 1)])
def test_generator_meets_spec(n, seed):
    m = system.generate(n, seed)
    x = m.xyz.astype(np.float64)
    b = np.linalg.norm(x[1:] - x[:-1], axis=1)
    assert np.abs(b - 3.8).max() < 1e-5
    u1, u2 = x[:-2] - x[1:-1], x[2:] - x[1:-1]
    ang = np.degrees(np.arccos((u1 * u2).sum(1) / np.linalg.norm(u1, axis=1) / np.linalg.norm(u2, axis=1)))
    assert ang.min() >= 80.0 - 1e-3 and ang.max() <= 150.0 + 1e-3
    R = 3.8 * n ** (1 / 3) * 1.2
    assert np.linalg.norm(x, axis=1).max() <= R + 1e-4
    if n <= 4000:
        d = np.sqrt(((x[:, None, :] - x[None, :, :]) ** 2).sum(-1))
        iu = np.triu_indices(n, 2)
        assert d[iu].min() >= 4.0 - 1e-4
        iu3 = np.triu_indices(n, 3)
        nat = set(zip(*[a[d[iu3] < 8.0] for a in iu3]))
        assert nat == set(zip(m.nat_i.tolist(), m.nat_j.tolist()))
    np.testing.assert_array_equal(m.bond_r0, np.linalg.norm(x[1:] - x[:-1], axis=1).astype(np.float32))


def test_generator_is_deterministic_and_seeded():
    a, b, c = system.generate(500, 7), system.generate(500, 7), system.generate(500, 8)
    np.testing.assert_array_equal(a.xyz, b.xyz)
    assert not np.array_equal(a.xyz, c.xyz)


def test_per_contact_epsilon_range():
    m = system.generate(2000, 2, (0.7, 1.3))
    assert m.nat_eps.min() >= 0.7 and m.nat_eps.max() <= 1.3
    assert m.nat_eps.std() > 0.1


def test_ensemble_and_requests_spec():
    ns, ts = system.ensemble_spec(512, 60, 1500, 0.5, 0.8, 4)
    assert ns.min() >= 60 and ns.max() <= 1500 and ts.min() >= 0.5 and ts.max() <= 0.8
    lg = np.log(ns)
    assert abs(lg.mean() - 0.5 * (np.log(60) + np.log(1500))) < 0.15
    r = system.request_stream(200.0, 5.0, seed=5)
    k = len(r["n"])
    assert 800 < k < 1200
    assert r["n"].min() >= 50 and r["n"].max() <= 20000
    assert r["steps"].min() >= 1e4 and r["steps"].max() <= 1e6
    assert np.all(np.diff(r["arrival"]) > 0)
    assert set(np.unique(r["extended"])) == {0, 1}


def test_philox_known_answers():
    """Philox4x32-10 known-answer vectors of the algorithm's reference release."""
    assert [hex(v) for v in O.philox([0, 0, 0, 0], [0, 0])] == \
        ["0x6627e8d5", "0xe169c58d", "0xbc57ac4c", "0x9b00dbd8"]
    assert [hex(v) for v in O.philox([0xffffffff] * 4, [0xffffffff] * 2)] == \
        ["0x408f276d", "0x41c83b0e", "0xa20bc7c6", "0x6d5451fd"]
    assert [hex(v) for v in O.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                                     [0xa4093822, 0x299f31d0])] == \
        ["0xd16cfe09", "0x94fdcceb", "0x5001e420", "0x24126ea1"]


def test_noise_normals_statistics():
    z = O.noise_normals(20000, 17, 3, 99)
    assert abs(z.mean()) < 0.02 and abs(z.std() - 1.0) < 0.02
    z2 = O.noise_normals(20000, 18, 3, 99)
    assert abs(np.corrcoef(z.ravel(), z2.ravel())[0, 1]) < 0.02


def test_oracle_pair_list_is_subset_of_neighbour_list():
    m = system.generate(600, 3)
    rng = np.random.default_rng(0)
    x = (m.xyz + rng.normal(0, 0.5, m.xyz.shape)).astype(np.float32)
    ni, nj = O.nl_rep(m, x, 3.2, 0.0)
    pi, pj = O.filter_rep(m, x, ni, nj, 2.5, 0.0)
    s_nl = set(zip(ni.tolist(), nj.tolist()))
    s_pl = set(zip(pi.tolist(), pj.tolist()))
    assert s_pl <= s_nl and len(s_pl) > 0
    nat = set(zip(m.nat_i.tolist(), m.nat_j.tolist()))
    assert not (s_nl & nat)
    assert all(j - i > 2 for i, j in s_nl)


def test_rcut_matches_reference_rounding():
    # rcut = 3.2 * r0 in double rounded to FP32, squared in FP32 (sop.cu:746-747)
    r0 = np.float32(5.123456)
    rc = np.float32(3.2 * np.float64(r0))
    assert O.lib().orc_rcut2(3.2, 0.0, r0) == np.float32(rc * rc)
    assert O.lib().orc_rcut2(0.0, 32.0, r0) == np.float32(1024.0)


def test_dropin_program_links_and_reaches_the_engine(tmp_path):
    """Where build() found a reference tree, it linked the reference program
    over the engine (sop_gb300/shim/build_shim_ref.sh).  Run here, without a
    GPU, the reference's own parser and loaders read an input script and the
    first replaced call, alloc_GPU_arrays, runs the shim, which reports that
    there is no device to create the engine's context on."""
    import subprocess
    exe = os.path.join(ROOT, "sop_gb300", "shim", "_build", "sop2_gb300.x")
    if not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libsopref.so")):
        pytest.skip("no reference tree was present at build time")
    assert os.path.exists(exe), "build() built oracle/_ref but not the drop-in program"
    from sop_gb300 import system
    mol = system.generate(32, 1)
    system.write_reference_files(mol, str(tmp_path / "m"))
    (tmp_path / "input").write_text(
        "set dynamics underdamped;\nset temp 0.6;\nset nstep 10;\nset nup 5;\n"
        "set cutofftype neighborlist;\n" +
        "".join(f"load {k} {tmp_path / 'm'}.{k};\n" for k in ("bonds", "angles", "vdw", "init")) +
        "run;\n")
    r = subprocess.run([exe, "input"], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert "[Finished reading initial coordinates (32)]" in r.stdout
    if r.returncode != 0:   # no device here: the shim's device query or the engine refuses
        assert "sop_ctx_create failed" in r.stderr or "cudaGetDevice failed" in r.stderr, r.stderr


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("parts", [1, 2, 3, 5])
def test_ensemble_split_by_beads(seed, parts):
    """The cut of an ensemble into contexts: contiguous, non-empty runs in id
    order, at most `parts` of them, each within one molecule of an equal
    share of the beads."""
    rng = np.random.default_rng(seed)
    sizes = [int(x) for x in rng.integers(10, 1500, size=int(rng.integers(1, 40)))]
    cuts = engine.split_by_beads(sizes, parts)
    assert cuts[0] == 0 and cuts[-1] == len(sizes)
    assert all(a < b for a, b in zip(cuts, cuts[1:]))
    assert len(cuts) - 1 == min(parts, len(sizes)) or len(cuts) - 1 < parts
    total, share = sum(sizes), sum(sizes) / parts
    acc = np.cumsum([0] + sizes)
    for k, c in enumerate(cuts[1:-1], start=1):
        # run k closes at the first molecule reaching k shares
        assert acc[c] >= k * share and acc[c - 1] < k * share
    assert engine.split_by_beads([], parts) == [0, 0]
    assert engine.split_by_beads([10, 10, 10], 10) == [0, 1, 2, 3]
    assert total == acc[-1]


def test_ensemble_refuses_what_it_cannot_run():
    """parts < 1, the persistent step form beside other contexts, and
    molecules added after commit (no GPU needed for the checks)."""
    with pytest.raises(ValueError):
        engine.Ensemble(engine.default_params(), parts=0)
    with pytest.raises(ValueError):
        engine.Ensemble(engine.default_params(step_split=3), parts=2)
    ens = engine.Ensemble(engine.default_params(step_split=3), parts=1)
    m = system.generate(60, 0)
    assert ens.add(m) == 0 and ens.add(m, m.xyz, T=0.7, traj=1) == 1
    ens.engines = [object()]     # as after commit
    with pytest.raises(RuntimeError):
        ens.add(m)


def test_ensemble_matched_params():
    """The contexts after the first take its lanes per bead and step form,
    without the size-bucket tiles; a tiled or one-block choice leaves the
    parameters as they were; the caller's window and every other field are
    kept."""
    p = engine.default_params(step_window=-1, h=0.03)
    tuned = {"lanes_per_bead": 8, "form": 2, "window": 0, "buckets": {"tiled": False}}
    q = engine.matched_params(p, tuned)
    assert (q.lanes_per_bead, q.step_split, q.step_buckets) == (8, 2, -1)
    assert (q.step_window, q.h, q.nnlup) == (-1, 0.03, p.nnlup)
    assert (p.lanes_per_bead, p.step_split, p.step_buckets) == (0, 0, 0)   # a copy
    q = engine.matched_params(p, dict(tuned, buckets={"tiled": True}))
    assert bytes(q) == bytes(p)
    q = engine.matched_params(p, dict(tuned, form=4))
    assert bytes(q) == bytes(p)


def test_ensemble_routes_ids_and_rows(monkeypatch):
    """Host logic of engine.Ensemble with a stand-in context class: molecule
    ids map to (context, local id) in id order, downloads of every bead land
    in each context's rows of the caller's array, and the contexts after the
    first are created with the first one's lanes and form."""
    made = []

    class FakeEngine:
        def __init__(self, params):
            self.params = engine.Params.from_buffer_copy(params)
            self.mols, self.tags = [], []
            made.append(self)

        def add(self, mol, xyz=None, **kw):
            self.mols.append(mol)
            self.tags.append(kw["traj"])
            return len(self.mols) - 1

        def commit(self):
            pass

        def tuning(self):
            return {"lanes_per_bead": 16, "form": 2, "window": 0, "buckets": {"tiled": False}}

        def status(self, i):
            return (0, 1000 * len(made) + self.tags[i])

        def download_all(self, out):
            assert out.flags.c_contiguous and out.shape == (sum(m.n for m in self.mols), 3)
            out[:] = np.repeat(np.array(self.tags, np.float32), [m.n for m in self.mols])[:, None]
            return out

        def close(self):
            pass

    monkeypatch.setattr(engine, "Engine", FakeEngine)
    sizes = [30, 200, 50, 400, 10, 90, 300]
    mols = [system.generate(n, k) for k, n in enumerate(sizes)]
    ens = engine.Ensemble(engine.default_params(), parts=3)
    for k, m in enumerate(mols):
        assert ens.add(m, m.xyz, T=0.6, traj=k) == k
    ens.commit()
    assert ens.cuts == engine.split_by_beads(sizes, 3) and len(made) == 3
    assert [t for e in made for t in e.tags] == list(range(len(mols)))
    assert (made[0].params.lanes_per_bead, made[0].params.step_split) == (0, 0)
    for e in made[1:]:
        assert (e.params.lanes_per_bead, e.params.step_split, e.params.step_buckets) == (16, 2, -1)
    for k in range(len(mols)):
        ctx = next(c for c in range(3) if ens.cuts[c] <= k < ens.cuts[c + 1])
        assert ens.status(k) == (0, 1000 * len(made) + k) and ens._where[k][0] == ctx
    allx = ens.download_all()
    np.testing.assert_array_equal(allx[:, 0], np.repeat(np.arange(len(mols), dtype=np.float32), sizes))
    with pytest.raises(RuntimeError):
        ens.commit()
    ens.close()
