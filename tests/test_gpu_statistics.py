"""Long runs compared with the reference.

Same noise: the engine and the oracle's serial FP32 run of the reference
loop (orc_ref_*: the reference's step order, sop.cu:197-278, with the same
Philox stream) start from the same structure; their trajectories agree to
FP32 rounding for the first hundred steps and only then drift apart
(molecular dynamics is chaotic).

Independent seeds, against the reference program itself: the reference's
own binary (underdamped_ctrl with cuRAND XORWOW noise, GPU list drivers) ran
its input script once per seed on the GPU (tests/golden/make_ref_stats.py;
ref_stats.npz holds each run's time averages of rna_etot, Rg^2, Q and the
kinetic temperature over steps 1,100 .. 5,000, sampled every 100 steps).  The
engine runs the same structures in the reference's settings -- factor-mode
cut-offs, neighbour list every 50 steps, pair list every step, kBT 0.6, the
reference's native energy coefficient 0.7 -- with one Philox stream per seed
and the same sampling.  Per observable, z = (mean_engine - mean_reference) /
combined standard error of the per-run means must satisfy |z| <= 2 (the
stated criterion); the kinetic temperature must agree within 1%.

Rg^2 is measured on both sides with the reference's own estimator: the
reference sums the squared distances of all N^2/2 pairs in float
(sop.cu:563-580), and for 4,000 beads that sum of 8 million positive terms
sits 0.4% below the exact value, about 3 standard errors of the 144-run
means.  The engine's samples are put through the oracle's bit-exact
restatement of that sum (orc_ref_rgsq, pinned in test_golden against the
reference's values), so the comparison is of dynamics, not of summation
order.

At h = 0.05 a FENE bond occasionally overshoots R0 in a long 4,000-bead run:
3 of the reference's 48 runs produced a NaN energy (log of a negative
argument, energy.cu:217-223) and one of them blew up.  The engine stops such
a molecule with SOP_MOL_FENE_RANGE.  Runs that failed are left out on both
sides, and the numbers of failed runs must agree within binomial noise.
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from oracle import pyoracle as O
from sop_gb300 import engine, system

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
T = 0.6
CUT = [0.0, 32.0, 0.0, 32.0, 0.0, 16.0, 0.0, 16.0]   # the engine's baseline cut-offs (A)
STATS = {"n128": (128, 0), "n4000": (4000, 1)}


def engine_means(mol, runs, equil, every, samples, boxl=500.0):
    """Per-run time averages of (rna_etot, Rg^2, Q, kinT) in the reference's
    settings, one batched context, one Philox stream per run.  Rg^2 is the
    reference's float estimator on each sampled frame (O.ref_rgsq), computed
    on a pool of host threads while the engine runs on."""
    p = engine.default_params(h=0.05, zeta=0.05, nnlup=50, nplup=1, seed=20240, boxl=boxl)
    eps_e = np.full(len(mol.nat_i), 0.7, np.float32)   # coeff_att[1][1] (global.cpp:51-55)
    e = engine.Engine(p)
    for k in range(runs):
        e.add(mol, mol.xyz, T=T, traj=k, eps_energy=eps_e)
    e.commit()
    e.step(equil)
    acc = np.zeros((runs, 4))
    O.lib()
    with ThreadPoolExecutor(os.cpu_count() or 4) as pool:
        rg = []
        for _ in range(samples):
            e.step(every)
            frame = e.download_all().reshape(runs, mol.n, 3)
            rg += [pool.submit(O.ref_rgsq, frame[m], boxl) for m in range(runs)]
            for m in range(runs):
                ob = e.observables(m)
                acc[m] += (e.energy(m)[4], 0.0, ob["Q"], ob["kinT"])
        acc[:, 1] = np.array([f.result() for f in rg]).reshape(samples, runs).sum(0)
    failed = np.array([e.status(m)[0] != 0 for m in range(runs)])
    e.close()
    acc /= samples
    acc[failed] = np.nan
    return acc


@pytest.mark.parametrize("name", list(STATS))
def test_long_runs_match_the_reference_program_within_2_sigma(name):
    path = os.path.join(GOLD, "ref_stats.npz")
    if not os.path.exists(path):
        pytest.skip("ref_stats.npz not generated")
    g = np.load(path)
    ref = g[f"{name}.means"]
    n, seed = STATS[name]
    equil, every = int(g["equil"]), int(g["nup"])
    samples = (int(g["nstep"]) - equil) // every
    eng = engine_means(system.generate(n, seed), len(ref), equil, every, samples)
    ok_e = np.isfinite(eng).all(1)
    ok_r = np.isfinite(ref).all(1) & (ref[:, 3] < 10 * T)
    fe, fr, nr = int((~ok_e).sum()), int((~ok_r).sum()), len(ref)
    pool = (fe + fr) / (2.0 * nr)
    print(name, "failed runs: engine", fe, "reference", fr, "of", nr)
    assert abs(fe - fr) <= 3.0 * np.sqrt(2.0 * nr * pool * (1.0 - pool)) + 1.0, (fe, fr)
    eng, ref = eng[ok_e], ref[ok_r]
    zs = {}
    for c, label in enumerate(("energy", "rgsq", "Q")):
        se = np.sqrt(eng[:, c].var(ddof=1) / len(eng) + ref[:, c].var(ddof=1) / len(ref))
        zs[label] = (eng[:, c].mean() - ref[:, c].mean()) / se
    print(name, "z (engine - reference) / se:", {k: round(float(v), 2) for k, v in zs.items()},
          "means engine", eng.mean(0).round(4), "reference", ref.mean(0).round(4))
    for label, z in zs.items():
        assert abs(z) <= 2.0, (name, label, z)
    ke, kr = eng[:, 3].mean(), ref[:, 3].mean()
    assert abs(ke - kr) < 0.01 * kr, (ke, kr)


def test_same_noise_tracks_the_reference_loop():
    mol = system.generate(128, 0)
    for traj in (0, 5):
        e = engine.plain(mol, mol.xyz, engine.baseline_params(seed=1234), T=T, traj=traj)
        r = O.RefRun(mol, mol.xyz, CUT, 0.05, 0.05, T, 50, 10, 1234, traj)
        r.advance(0)
        done = 0
        for k in (1, 10, 50, 100):
            e.step(k - done)
            r.advance(k - done)
            done = k
            g, c = e.download(), r.state()
            dx = np.abs(g["unc_pos"] - c["unc_pos"]).max()
            dv = np.abs(g["vel"] - c["vel"]).max()
            assert dx < 1e-4 and dv < 1e-3, (traj, k, dx, dv)
        e.close()
        r.close()


@pytest.mark.parametrize("name,n,seed,slope", [("n128", 128, 0, 2e-6), ("n4000", 4000, 1, 5e-6)])
def test_same_noise_tracks_the_reference_program(name, n, seed, slope):
    """The engine against the reference program itself, step for step, on the
    reference's own noise: the reference built with its host generator ran
    with `set run 7` and wrote its coordinates after every step
    (tests/golden/make_ref_traj.py); the engine takes the same deviates
    (orc_ref_gasdev, the oracle's bit-exact restatement of that generator)
    as injected noise, one set of 3 per bead per force evaluation, in the
    reference's order.  The trajectories agree to FP32 rounding, which grows
    slowly (the writer's 6 decimals are the floor): max |dx| <= 2e-5 +
    slope * step, for 300 steps at 128 beads and 100 at 4,000."""
    path = os.path.join(GOLD, "ref_traj.npz")
    if not os.path.exists(path):
        pytest.skip("ref_traj.npz not generated")
    g = np.load(path)
    steps, frames = g[f"{name}.steps"], g[f"{name}.unc"]
    mol = system.generate(n, seed)
    last = int(steps.max())
    noise = O.ref_gasdev(int(g["run"]), 3 * n * (last + 1)).reshape(last + 1, n, 3)
    noise = noise.astype(np.float32)
    p = engine.default_params(h=0.05, zeta=0.05, nnlup=50, nplup=1)
    with engine.plain(mol, mol.xyz, p, T=T) as e:
        e.set_noise(noise[0])
        e.force_eval()           # the set-up's force evaluation (sop.cu:180-186)
        want = dict(zip(steps.tolist(), frames))
        worst = {}
        for k in range(1, last + 1):
            e.set_noise(noise[k])
            e.step(1)
            if k in want:
                worst[k] = float(np.abs(e.download()["unc_pos"] - want[k]).max())
    print(name, {k: f"{v:.1e}" for k, v in worst.items()})
    for k, v in worst.items():
        assert v <= 2e-5 + slope * k, (name, k, v)
