"""sop_energy_noalloc: the energy reduction for callers that may not allocate
device memory (an application whose own memory manager owns the device, a
loop that must not stall on an allocation's implicit synchronisation).  The
caller owns every input and output buffer; the entry point keeps its partial
sums in a fixed device array of the library.

Checked through the C ABI against sop_energy on the same coordinates and
lists, on two calls in a row (the shared scratch keeps the previous call's
contents, which must not leak into the next result).  This file is collected
last so that a run stopping at the first failure has run every other test.
"""
import numpy as np
import pytest

from sop_gb300 import engine, system

pytestmark = pytest.mark.gpu

ENERGY_RTOL = 2e-5   # the tolerance of the energy parity tests


def _device(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a, dtype)).cuda()


def _lists(torch, e, mol, keep, eps_energy="force"):
    """Coordinates and the context's current lists in caller-owned device
    memory.  eps_energy: "force" passes mol.nat_eps as the native energy
    epsilons, None passes NULL (1.0), an array passes those values."""
    d = e.download(0)
    key = {}
    for k, (a, b) in enumerate(zip(mol.nat_i, mol.nat_j)):
        key[(int(a), int(b))] = key[(int(b), int(a))] = k
    ai, aj, ar = e.list_pairs(0, 2)
    src = mol.nat_eps if isinstance(eps_energy, str) else eps_energy
    aeps = None if src is None else \
        np.array([src[key[(int(a), int(b))]] for a, b in zip(ai, aj)], np.float32)
    ri, rj, _ = e.list_pairs(0, 3)
    t = dict(x=_device(torch, d["unc_pos"], np.float32),
             ty=None if mol.types is None else _device(torch, mol.types, np.int32), bi=_device(torch, mol.bond_i, np.int32),
             bj=_device(torch, mol.bond_j, np.int32), br=_device(torch, mol.bond_r0, np.float32),
             ai=_device(torch, mol.ang_i, np.int32), ak=_device(torch, mol.ang_k, np.int32),
             pi=_device(torch, ai, np.int32), pj=_device(torch, aj, np.int32),
             pr=_device(torch, ar, np.float32),
             pe=None if aeps is None else _device(torch, aeps, np.float32),
             ri=_device(torch, ri, np.int32), rj=_device(torch, rj, np.int32))
    keep.append(t)
    p = lambda k: t[k].data_ptr()  # noqa: E731
    ty = None if t["ty"] is None else p("ty")
    pe = None if t["pe"] is None else p("pe")
    return engine.EnergyLists(mol.n, p("x"), ty, len(mol.bond_i), p("bi"), p("bj"), p("br"),
                              len(mol.ang_i), p("ai"), p("ak"), len(ai), p("pi"), p("pj"),
                              p("pr"), pe, len(ri), p("ri"), p("rj"))


def _twice(torch, params, lists, ref, out):
    for _ in range(2):
        out.fill_(float("nan"))
        engine.energy_noalloc(params, lists, out.data_ptr(), 0)
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=ENERGY_RTOL, atol=1e-6)


def test_noalloc_energy_matches_sop_energy_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    params = engine.baseline_params()
    keep = []
    mols = [system.generate(1500, 21), system.generate(300, 22, (0.7, 1.3))]
    rng = np.random.default_rng(4)
    mols[1].types = rng.integers(1, 3, mols[1].n).astype(np.int32)   # two bead types
    out = torch.empty(5, dtype=torch.float64, device="cuda")
    for mol in mols:
        x = (mol.xyz + rng.normal(0.0, 0.2, mol.xyz.shape)).astype(np.float32)
        with engine.plain(mol, x, params, T=0.6) as e:
            ref = e.energy(0)
            lists = _lists(torch, e, mol, keep)
        _twice(torch, params, lists, ref, out)


def test_noalloc_energy_epsilons_default_and_energy_specific():
    """att_eps NULL means 1.0 for every native pair (checked on a molecule
    whose epsilons are all 1.0); a context whose native energy epsilons differ
    from its force epsilons is matched when the call gets the energy ones."""
    torch = pytest.importorskip("torch")
    params = engine.baseline_params()
    keep = []
    out = torch.empty(5, dtype=torch.float64, device="cuda")
    rng = np.random.default_rng(8)
    unit = system.generate(400, 23)
    assert np.all(unit.nat_eps == 1.0)
    x = (unit.xyz + rng.normal(0.0, 0.2, unit.xyz.shape)).astype(np.float32)
    with engine.plain(unit, x, params, T=0.6) as e:
        ref = e.energy(0)
        lists = _lists(torch, e, unit, keep, eps_energy=None)
    _twice(torch, params, lists, ref, out)
    mol = system.generate(400, 24, (0.7, 1.3))
    eps_e = rng.uniform(0.5, 1.5, len(mol.nat_i)).astype(np.float32)
    x = (mol.xyz + rng.normal(0.0, 0.2, mol.xyz.shape)).astype(np.float32)
    with engine.plain(mol, x, params, T=0.6, eps_energy=eps_e) as e:
        ref = e.energy(0)
        force_eps_lists = _lists(torch, e, mol, keep)
        lists = _lists(torch, e, mol, keep, eps_energy=eps_e)
    _twice(torch, params, lists, ref, out)
    engine.energy_noalloc(params, force_eps_lists, out.data_ptr(), 0)
    torch.cuda.synchronize()
    assert abs(out.cpu().numpy()[2] - ref[2]) > 1e-3   # the epsilons do matter


def test_noalloc_bad_index_gives_nan_not_a_read():
    """A native pair naming bead nbead (one past the end) is skipped by the
    kernel's own bounds check: its term and the total come back NaN, the other
    terms are unchanged, and a following valid call is exact again."""
    torch = pytest.importorskip("torch")
    params = engine.baseline_params()
    keep = []
    out = torch.empty(5, dtype=torch.float64, device="cuda")
    mol = system.generate(200, 25)
    with engine.plain(mol, mol.xyz, params, T=0.6) as e:
        ref = e.energy(0)
        lists = _lists(torch, e, mol, keep)
    bad_j = keep[-1]["pj"].clone()
    bad_j[0] = mol.n
    keep.append(bad_j)
    bad = engine.EnergyLists(*[getattr(lists, f) for f, _ in engine.EnergyLists._fields_])
    bad.att_j = bad_j.data_ptr()
    out.fill_(0.0)
    engine.energy_noalloc(params, bad, out.data_ptr(), 0)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.isnan(got[2]) and np.isnan(got[4])
    np.testing.assert_allclose(got[[0, 1, 3]], ref[[0, 1, 3]], rtol=ENERGY_RTOL, atol=1e-6)
    _twice(torch, params, lists, ref, out)


def test_noalloc_rejects_inputs_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    params = engine.baseline_params()
    x = torch.zeros(3 * 8, dtype=torch.float32, device="cuda")
    idx = torch.zeros(8, dtype=torch.int32, device="cuda")
    out = torch.zeros(5, dtype=torch.float64, device="cuda")
    lists = engine.EnergyLists(8, x.data_ptr(), None, 0, None, None, None, 0, None, None, 0, None,
                               None, None, None, engine.ENERGY_NOALLOC_MAX_ITEMS + 1,
                               idx.data_ptr(), idx.data_ptr())
    with pytest.raises(engine.SopError) as ei:
        engine.energy_noalloc(params, lists, out.data_ptr(), 0)
    assert ei.value.code == 4  # SOP_ERR_CAPACITY, refused before any launch
