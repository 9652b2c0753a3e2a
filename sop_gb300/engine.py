"""Python binding of libsopgpu.so (include/sop_gpu.h) through ctypes.

This is a thin host-side mirror of the engine's C ABI; every computation runs
in the CUDA library.  Importing works without a GPU; creating a context
requires the built library and a CUDA device and raises otherwise -- there is
no CPU fallback.

Reference correspondence (samchogroup/SOP):
  Engine(...) + add()/commit()  alloc_GPU_arrays, setup_rng, initial lists and
                                force_eval of underdamped_ctrl (sop.cu:133-186)
  step(n)                       the loop body of underdamped_ctrl (sop.cu:197-243)
  update_neighbor_list()        update_neighbor_list (sop.cu:928-1262)
  update_pair_list()            update_pair_list (sop.cu:1456-1706)
  force_eval()                  force_eval (energy.cu:81-150)
  energy()                      energy_eval (energy.cu:69-78)
  observables()                 calculate_observables (sop.cu:528-611)
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .system import Molecule

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

SOP_OK = 0
STATUS_NAMES = {1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_ALLOC", 4: "ERR_CAPACITY",
                5: "ERR_MOLECULE", 6: "ERR_BUDGET", 7: "ERR_NOT_FOUND"}
MOL_FENE_RANGE, MOL_NONFINITE, MOL_DONE = 1, 2, 4


class SopError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class Params(ctypes.Structure):
    _fields_ = [("k_bnd", ctypes.c_double), ("R0", ctypes.c_double),
                ("eps_ss", ctypes.c_double), ("sigma_ss", ctypes.c_double),
                ("eps_rep", ctypes.c_double), ("boxl", ctypes.c_double),
                ("h", ctypes.c_double), ("zeta", ctypes.c_double),
                ("nl_att_fac", ctypes.c_double), ("nl_att_abs", ctypes.c_double),
                ("nl_rep_fac", ctypes.c_double), ("nl_rep_abs", ctypes.c_double),
                ("pl_att_fac", ctypes.c_double), ("pl_att_abs", ctypes.c_double),
                ("pl_rep_fac", ctypes.c_double), ("pl_rep_abs", ctypes.c_double),
                ("nnlup", ctypes.c_int), ("nplup", ctypes.c_int), ("rep6", ctypes.c_int),
                ("device", ctypes.c_int), ("graph_steps", ctypes.c_int),
                ("lanes_per_bead", ctypes.c_int), ("seed", ctypes.c_ulonglong),
                ("integrator", ctypes.c_int), ("step_split", ctypes.c_int),
                ("step_window", ctypes.c_int), ("step_buckets", ctypes.c_int),
                ("nl_rows", ctypes.c_int)]


class MoleculeDesc(ctypes.Structure):
    _fields_ = [("nbead", ctypes.c_int),
                ("nbnd", ctypes.c_int), ("bond_i", ctypes.c_void_p), ("bond_j", ctypes.c_void_p),
                ("bond_r0", ctypes.c_void_p),
                ("nang", ctypes.c_int), ("ang_i", ctypes.c_void_p), ("ang_k", ctypes.c_void_p),
                ("nnat", ctypes.c_int), ("nat_i", ctypes.c_void_p), ("nat_j", ctypes.c_void_p),
                ("nat_r0", ctypes.c_void_p), ("nat_eps", ctypes.c_void_p),
                ("nat_eps_energy", ctypes.c_void_p), ("types", ctypes.c_void_p),
                ("unc_pos", ctypes.c_void_p), ("pos", ctypes.c_void_p), ("vel", ctypes.c_void_p),
                ("T", ctypes.c_double), ("traj", ctypes.c_uint), ("nsteps", ctypes.c_longlong)]


class EnergyLists(ctypes.Structure):
    """sop_energy_lists: device pointers owned by the caller."""
    _fields_ = [("nbead", ctypes.c_int), ("unc_pos", ctypes.c_void_p), ("types", ctypes.c_void_p),
                ("nbnd", ctypes.c_int), ("bond_i", ctypes.c_void_p), ("bond_j", ctypes.c_void_p),
                ("bond_r0", ctypes.c_void_p),
                ("nang", ctypes.c_int), ("ang_i", ctypes.c_void_p), ("ang_k", ctypes.c_void_p),
                ("natt", ctypes.c_int), ("att_i", ctypes.c_void_p), ("att_j", ctypes.c_void_p),
                ("att_r0", ctypes.c_void_p), ("att_eps", ctypes.c_void_p),
                ("nrep", ctypes.c_longlong), ("rep_i", ctypes.c_void_p), ("rep_j", ctypes.c_void_p)]


ENERGY_NOALLOC_MAX_ITEMS = 4194304


def energy_noalloc(params: "Params", lists: EnergyLists, terms_ptr: int, stream: int = 0) -> None:
    """sop_energy_noalloc: energy terms of caller-owned device lists into the
    caller-owned device array at terms_ptr (5 doubles); allocates nothing."""
    rc = lib().sop_energy_noalloc(ctypes.byref(params), ctypes.byref(lists),
                                  ctypes.c_void_p(terms_ptr), ctypes.c_void_p(stream))
    if rc != SOP_OK:
        raise SopError(rc, (lib().sop_energy_noalloc_error() or b"").decode())


def lib_path() -> str:
    return os.path.join(_HERE, "libsopgpu.so")


def lib() -> ctypes.CDLL:
    """The engine library; raises if it was not built (no fallback exists)."""
    global _LIB
    if _LIB is None:
        p = lib_path()
        if not os.path.exists(p):
            raise RuntimeError(f"{p} is missing: the CUDA engine must be built "
                               "(python -c 'import __graft_entry__ as g; g.build()')")
        L = ctypes.CDLL(p)
        V, I, LL = ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong
        PLL = ctypes.POINTER(LL)
        sig = {
            "sop_params_default": (None, [ctypes.POINTER(Params)]),
            "sop_ctx_create": (I, [ctypes.POINTER(Params), ctypes.POINTER(V)]),
            "sop_ctx_destroy": (I, [V]),
            "sop_add_molecule": (I, [V, ctypes.POINTER(MoleculeDesc), ctypes.POINTER(I)]),
            "sop_commit": (I, [V]),
            "sop_upload_topology": (I, [V, ctypes.POINTER(MoleculeDesc)]),
            "sop_upload_state": (I, [V, I, V, V, V]),
            "sop_step": (I, [V, LL]),
            "sop_step_async": (I, [V, LL]),
            "sop_sync": (I, [V]),
            "sop_launch_stage": (I, [V, I, I]),
            "sop_update_neighbor_list": (I, [V, PLL, PLL]),
            "sop_update_pair_list": (I, [V, PLL, PLL]),
            "sop_force_eval": (I, [V]),
            "sop_set_noise": (I, [V, V]),
            "sop_download": (I, [V, I, V, V, V, V]),
            "sop_download_list": (I, [V, I, I, LL, V, V, V, PLL]),
            "sop_list_sizes": (I, [V, V]),
            "sop_download_all": (I, [V, V]),
            "sop_download_all_async": (I, [V, V, PLL]),
            "sop_download_wait": (I, [V, LL]),
            "sop_energy": (I, [V, I, V]),
            "sop_observables": (I, [V, I, V]),
            "sop_molecule_status": (I, [V, I, ctypes.POINTER(I), PLL]),
            "sop_memory": (I, [V, I, PLL, PLL]),
            "sop_tuning": (I, [V, ctypes.POINTER(I), V]),
            "sop_stream": (I, [V, ctypes.POINTER(V)]),
            "sop_last_error": (ctypes.c_char_p, [V]),
            "sop_serve_create": (I, [ctypes.POINTER(Params), LL, LL, ctypes.POINTER(V)]),
            "sop_serve_submit": (I, [V, ctypes.POINTER(MoleculeDesc), ctypes.POINTER(I)]),
            "sop_serve_advance": (I, [V, I]),
            "sop_serve_finished": (I, [V, I, V, ctypes.POINTER(I)]),
            "sop_serve_result": (I, [V, I, V, V, V, ctypes.POINTER(I), PLL,
                                     ctypes.POINTER(ctypes.c_double)]),
            "sop_serve_stats": (I, [V, V]),
            "sop_step_form": (I, [V, ctypes.POINTER(I), ctypes.POINTER(I)]),
            "sop_step_window": (I, [V, ctypes.POINTER(I)]),
            "sop_step_buckets": (I, [V, ctypes.POINTER(I), V, V, V, V]),
            "sop_check_step_barrier": (I, [V, I, ctypes.c_double, ctypes.POINTER(I)]),
            "sop_checkpoint": (I, [V, I, V, LL, PLL]),
            "sop_restore": (I, [V, I, V, LL]),
            "sop_serve_checkpoint": (I, [V, I, V, LL, PLL]),
            "sop_serve_resume": (I, [V, ctypes.POINTER(MoleculeDesc), V, LL, ctypes.POINTER(I)]),
            "sop_energy_noalloc": (I, [ctypes.POINTER(Params), ctypes.POINTER(EnergyLists), V, V]),
            "sop_energy_noalloc_error": (ctypes.c_char_p, []),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def default_params(**kw) -> Params:
    p = Params()
    lib().sop_params_default(ctypes.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def baseline_params(**kw) -> Params:
    """The synthetic workloads' settings: absolute 32 A / 16 A list cut-offs,
    neighbour list every 50 steps, pair list every 10, h = 0.05, zeta = 0.05."""
    base = dict(h=0.05, zeta=0.05, nl_att_fac=0.0, nl_att_abs=32.0, nl_rep_fac=0.0,
                nl_rep_abs=32.0, pl_att_fac=0.0, pl_att_abs=16.0, pl_rep_fac=0.0,
                pl_rep_abs=16.0, nnlup=50, nplup=10)
    base.update(kw)
    return default_params(**base)


_F32, _I32 = np.dtype(np.float32), np.dtype(np.int32)


def _arr(a, dt):
    """a as a C-contiguous array of dtype dt, without a copy when it is one."""
    if type(a) is np.ndarray and a.dtype == dt and a.flags.c_contiguous:
        return a
    return np.ascontiguousarray(a, dt)


def _addr(a):
    """The address of an array's data as an integer (None for None)."""
    if a is None:
        return None
    try:  # the buffer protocol: about a third of the cost of .ctypes
        return ctypes.addressof(ctypes.c_char.from_buffer(a))
    except (TypeError, ValueError, BufferError):  # read-only or empty arrays
        return a.ctypes.data


def _p(a):
    """The address of an array's data (None for None)."""
    if a is None:
        return None
    try:  # the buffer protocol: about a third of the cost of .ctypes
        return ctypes.c_void_p(ctypes.addressof(ctypes.c_char.from_buffer(a)))
    except (TypeError, ValueError, BufferError):  # read-only or empty arrays
        return ctypes.c_void_p(a.ctypes.data)


class Engine:
    """One context: one or more independent molecules on one GPU stream."""

    def __init__(self, params: Params | None = None):
        self._keep = []
        self.params = params if params is not None else default_params()
        h = ctypes.c_void_p()
        self._check(lib().sop_ctx_create(ctypes.byref(self.params), ctypes.byref(h)), None)
        self.h = h
        self.mols: list[Molecule] = []

    def _check(self, rc: int, h) -> None:
        if rc != SOP_OK:
            msg = lib().sop_last_error(h)
            raise SopError(rc, msg.decode() if msg else "")

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().sop_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def add(self, mol: Molecule, xyz: np.ndarray | None = None, T: float = 0.6, traj: int = 0,
            nsteps: int = -1, vel: np.ndarray | None = None, pos: np.ndarray | None = None,
            eps_energy: np.ndarray | None = None) -> int:
        # arrays already of the right type and layout are passed as they are
        # (the common case: the generator's), others converted; the
        # addresses go into the descriptor as plain integers
        f32, i32 = _F32, _I32
        x, bi, bj, br = _arr(mol.xyz if xyz is None else xyz, f32), _arr(mol.bond_i, i32), \
            _arr(mol.bond_j, i32), _arr(mol.bond_r0, f32)
        ai, ak = _arr(mol.ang_i, i32), _arr(mol.ang_k, i32)
        ni, nj, nr, ne = _arr(mol.nat_i, i32), _arr(mol.nat_j, i32), _arr(mol.nat_r0, f32), \
            _arr(mol.nat_eps, f32)
        ty = _arr(mol.types, i32)
        v = None if vel is None else _arr(vel, f32)
        ps = None if pos is None else _arr(pos, f32)
        ee = None if eps_energy is None else _arr(eps_energy, f32)
        d = MoleculeDesc(mol.n, len(bi), _addr(bi), _addr(bj), _addr(br), len(ai), _addr(ai),
                         _addr(ak), len(ni), _addr(ni), _addr(nj), _addr(nr), _addr(ne), _addr(ee),
                         _addr(ty), _addr(x), _addr(ps), _addr(v), float(T), int(traj), int(nsteps))
        mid = ctypes.c_int()
        self._check(lib().sop_add_molecule(self.h, ctypes.byref(d), ctypes.byref(mid)), self.h)
        self.mols.append(mol)
        return mid.value

    def commit(self) -> None:
        self._check(lib().sop_commit(self.h), self.h)

    def step(self, n: int) -> None:
        self._check(lib().sop_step(self.h, int(n)), self.h)

    def step_async(self, n: int) -> None:
        self._check(lib().sop_step_async(self.h, int(n)), self.h)

    def sync(self) -> None:
        self._check(lib().sop_sync(self.h), self.h)

    def launch_stage(self, stage: int, koff: int = 0) -> None:
        self._check(lib().sop_launch_stage(self.h, int(stage), int(koff)), self.h)

    def force_eval(self) -> None:
        self._check(lib().sop_force_eval(self.h), self.h)

    def set_noise(self, normals: np.ndarray | None) -> None:
        if normals is None:
            self._check(lib().sop_set_noise(self.h, None), self.h)
        else:
            z = np.ascontiguousarray(normals, np.float32)
            self._check(lib().sop_set_noise(self.h, _p(z)), self.h)

    def update_neighbor_list(self) -> tuple[int, int]:
        a, r = ctypes.c_longlong(), ctypes.c_longlong()
        self._check(lib().sop_update_neighbor_list(self.h, ctypes.byref(a), ctypes.byref(r)), self.h)
        return a.value, r.value

    def update_pair_list(self) -> tuple[int, int]:
        a, r = ctypes.c_longlong(), ctypes.c_longlong()
        self._check(lib().sop_update_pair_list(self.h, ctypes.byref(a), ctypes.byref(r)), self.h)
        return a.value, r.value

    def upload_state(self, mol: int, unc_pos, pos=None, vel=None) -> None:
        u = np.ascontiguousarray(unc_pos, np.float32)
        p = None if pos is None else np.ascontiguousarray(pos, np.float32)
        v = None if vel is None else np.ascontiguousarray(vel, np.float32)
        self._check(lib().sop_upload_state(self.h, mol, _p(p), _p(u), _p(v)), self.h)

    def download(self, mol: int = 0) -> dict:
        n = self.mols[mol].n
        out = {k: np.empty((n, 3), np.float32) for k in ("pos", "unc_pos", "vel", "force")}
        self._check(lib().sop_download(self.h, mol, _p(out["pos"]), _p(out["unc_pos"]),
                                       _p(out["vel"]), _p(out["force"])), self.h)
        return out

    def list_pairs(self, mol: int, which: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(i, j, r0) of a list: 0 att NL, 1 rep NL, 2 att PL, 3 rep PL."""
        cnt = ctypes.c_longlong()
        self._check(lib().sop_download_list(self.h, mol, which, 0, None, None, None,
                                            ctypes.byref(cnt)), self.h)
        k = cnt.value
        i, j = np.empty(max(k, 1), np.int32), np.empty(max(k, 1), np.int32)
        r0 = np.empty(max(k, 1), np.float32)
        self._check(lib().sop_download_list(self.h, mol, which, k, _p(i), _p(j), _p(r0),
                                            ctypes.byref(cnt)), self.h)
        return i[:k], j[:k], r0[:k]

    def list_sizes(self) -> dict:
        o = np.zeros(4, np.int64)
        self._check(lib().sop_list_sizes(self.h, _p(o)), self.h)
        return {"nnl_att": int(o[0]), "nnl_rep": int(o[1]), "nil_att": int(o[2]),
                "nil_rep": int(o[3])}

    def download_all(self, out: np.ndarray | None = None) -> np.ndarray:
        """Coordinates of every bead, molecules in id order, shape (total, 3)."""
        total = sum(m.n for m in self.mols)
        if out is None:
            out = np.empty((total, 3), np.float32)
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.size == 3 * total
        self._check(lib().sop_download_all(self.h, _p(out)), self.h)
        return out

    def download_all_async(self, out: np.ndarray) -> int:
        """Queues the copy of every bead's coordinates (as download_all, at the
        point the queued work will have reached) into `out` and returns a
        ticket for download_wait.  `out` should be page-locked (the call then
        returns at once) and must stay alive until the wait."""
        total = sum(m.n for m in self.mols)
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.size == 3 * total
        t = ctypes.c_longlong()
        self._check(lib().sop_download_all_async(self.h, _p(out), ctypes.byref(t)), self.h)
        self._inflight = getattr(self, "_inflight", {})
        self._inflight[t.value % 2] = out   # keeps the destination alive
        return t.value

    def download_wait(self, ticket: int) -> None:
        self._check(lib().sop_download_wait(self.h, int(ticket)), self.h)

    def energy(self, mol: int = 0) -> np.ndarray:
        t = np.zeros(5, np.float64)
        self._check(lib().sop_energy(self.h, mol, _p(t)), self.h)
        return t

    def checkpoint(self, mol: int = 0) -> bytes:
        """Exact checkpoint of a molecule (sop_checkpoint)."""
        size = ctypes.c_longlong()
        self._check(lib().sop_checkpoint(self.h, mol, None, 0, ctypes.byref(size)), self.h)
        buf = ctypes.create_string_buffer(size.value)
        self._check(lib().sop_checkpoint(self.h, mol, buf, size.value, ctypes.byref(size)), self.h)
        return buf.raw[:size.value]

    def restore(self, mol: int, blob: bytes) -> None:
        """Continue molecule `mol` from a checkpoint (sop_restore)."""
        self._check(lib().sop_restore(self.h, mol, blob, len(blob)), self.h)

    def observables(self, mol: int = 0) -> dict:
        o = np.zeros(4, np.float64)
        self._check(lib().sop_observables(self.h, mol, _p(o)), self.h)
        return {"Q": o[0], "rgsq": o[1], "kinT": o[2], "contct_nat": int(o[3])}

    def status(self, mol: int = 0) -> tuple[int, int]:
        st, step = ctypes.c_int(), ctypes.c_longlong()
        self._check(lib().sop_molecule_status(self.h, mol, ctypes.byref(st), ctypes.byref(step)),
                    self.h)
        return st.value, step.value

    def memory(self, mol: int = 0) -> tuple[int, int]:
        a, b = ctypes.c_longlong(), ctypes.c_longlong()
        self._check(lib().sop_memory(self.h, mol, ctypes.byref(a), ctypes.byref(b)), self.h)
        return a.value, b.value

    def tuning(self) -> dict:
        g = ctypes.c_int()
        ms = np.zeros(4, np.float32)
        self._check(lib().sop_tuning(self.h, ctypes.byref(g), _p(ms)), self.h)
        form = ctypes.c_int()
        self._check(lib().sop_step_form(self.h, None, ctypes.byref(form)), self.h)
        win = ctypes.c_int()
        self._check(lib().sop_step_window(self.h, ctypes.byref(win)), self.h)
        tiled = ctypes.c_int()
        bl, bf = np.zeros(3, np.int32), np.zeros(3, np.int32)
        bb, bms = np.zeros(3, np.int64), np.zeros(2, np.float32)
        self._check(lib().sop_step_buckets(self.h, ctypes.byref(tiled), _p(bl), _p(bf), _p(bb),
                                           _p(bms)), self.h)
        buckets = {"tiled": bool(tiled.value), "ms_tiled": float(bms[0]),
                   "ms_whole": float(bms[1]),
                   "by_bucket": {name: {"beads": int(bb[k]), "lanes_per_bead": int(bl[k]),
                                        "form": int(bf[k])}
                                 for k, name in enumerate(("<200", "200-599", ">=600"))}}
        return {"lanes_per_bead": g.value, "form": form.value, "window": win.value,
                "buckets": buckets,
                "ms": {str(k): float(v) for k, v in zip((2, 4, 8, 16), ms)}}

    def check_step_barrier(self, missing: int, timeout_s: float) -> bool:
        """Runs the persistent step's device-wide barrier with `missing`
        arrivals that never come; True when a wait ran out."""
        t = ctypes.c_int()
        self._check(lib().sop_check_step_barrier(self.h, int(missing), float(timeout_s),
                                                 ctypes.byref(t)), self.h)
        return bool(t.value)

    def stream(self) -> int:
        s = ctypes.c_void_p()
        self._check(lib().sop_stream(self.h, ctypes.byref(s)), self.h)
        return s.value or 0


def split_by_beads(sizes, parts: int) -> list[int]:
    """Cut points [0, c1, ..., len(sizes)] that split molecules of `sizes`
    beads (in id order) into at most `parts` contiguous, non-empty runs of
    about equal bead counts: run k closes after the first molecule at which
    the beads so far reach k/parts of the total."""
    n = len(sizes)
    parts = max(1, min(int(parts), n))
    total = int(sum(sizes))
    cuts, acc = [0], 0
    for i in range(n - 1):
        acc += int(sizes[i])
        if len(cuts) < parts and acc * parts >= len(cuts) * total:
            cuts.append(i + 1)
    cuts.append(n)
    return cuts


def matched_params(params: Params, tuned: dict) -> Params:
    """A copy of `params` fixed to the lanes per bead and the step form the
    tuner chose for a context (Engine.tuning()), without the size-bucket
    tiles.  Unchanged when it chose the tiles, which the parameters cannot
    fix, or the one-block form, which the tuner tries only for contexts of up
    to 2,048 beads.  The window stays as the parameters give it: the tuner uses
    one only where they fix it."""
    q = Params.from_buffer_copy(params)
    if not tuned["buckets"]["tiled"] and tuned["form"] in (1, 2):
        q.lanes_per_bead = tuned["lanes_per_bead"]
        q.step_split = tuned["form"]
        q.step_buckets = -1
    return q


class Ensemble:
    """A batched ensemble held as `parts` contexts (sop_ctx_create each), each
    on its own CUDA stream, stepped together.

    One context runs its kernels one after another: the list rebuilds, the
    tail of every launch and the gaps between launches leave SMs idle.  With
    two contexts on two streams the other context's kernels fill them (the
    512-trajectory ensemble: 3.06e9 bead-steps/s against 2.75e9 in one
    context on a GB300).

    Molecules keep the ids add() returns.  commit() gives each context a
    contiguous run of them, cut at equal bead counts (split_by_beads), so
    download_all() returns every bead in id order with one copy per context.
    A molecule's lists, noise (the Philox stream of its trajectory) and steps
    depend on its own beads alone, so every result is bit-identical to that of
    one context holding the whole ensemble.  The persistent step form
    (step_split 3) is refused for parts > 1: its device-wide barrier needs every
    block of its grid resident while another context's kernels run beside it.

    The first context is tuned alone; the others take its lanes per bead and
    step form (matched_params).  Contexts in different forms gain nothing (the ensemble
    above, both streams joined every 10 steps: 2.72e9 with one context in the
    one-kernel form and one in the two-kernel form, 2.95e9 with both in either
    form, 2.69e9 in one context).
    """

    def __init__(self, params: Params | None = None, parts: int = 2):
        self.params = params if params is not None else default_params()
        if int(parts) < 1:
            raise ValueError("parts must be at least 1")
        if int(parts) > 1 and self.params.step_split == 3:
            raise ValueError("the persistent step form (step_split 3) runs in one context only")
        self.parts = int(parts)
        self.mols: list[Molecule] = []
        self.engines: list[Engine] = []
        self._pending = []
        self._where: list[tuple[int, int]] = []   # molecule id -> (context, id in it)
        self.cuts: list[int] = []

    def add(self, mol: Molecule, xyz: np.ndarray | None = None, **kw) -> int:
        """Queues a molecule (the arguments of Engine.add); returns its id."""
        if self.engines:
            raise RuntimeError("add() after commit()")
        self._pending.append((mol, xyz, kw))
        self.mols.append(mol)
        return len(self.mols) - 1

    def commit(self) -> None:
        if self.engines:
            raise RuntimeError("commit() called twice")
        self.cuts = split_by_beads([m.n for m in self.mols], self.parts)
        params = self.params
        try:
            for c0, c1 in zip(self.cuts[:-1], self.cuts[1:]):
                e = Engine(params)
                self.engines.append(e)
                for i in range(c0, c1):
                    mol, xyz, kw = self._pending[i]
                    local = e.add(mol, xyz, **kw)
                    self._where.append((len(self.engines) - 1, local))
                e.commit()
                if len(self.engines) == 1:
                    params = matched_params(self.params, e.tuning())
        except Exception:
            self.close()
            raise
        self._pending = []

    def _at(self, mol: int) -> tuple[Engine, int]:
        k, local = self._where[mol]
        return self.engines[k], local

    def close(self) -> None:
        for e in self.engines:
            e.close()
        self.engines = []

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def step_async(self, n: int) -> None:
        for e in self.engines:
            e.step_async(n)

    def sync(self) -> None:
        for e in self.engines:
            e.sync()

    def step(self, n: int) -> None:
        self.step_async(n)
        self.sync()

    def streams(self) -> list[int]:
        return [e.stream() for e in self.engines]

    def status(self, mol: int = 0) -> tuple[int, int]:
        e, i = self._at(mol)
        return e.status(i)

    def download(self, mol: int = 0) -> dict:
        e, i = self._at(mol)
        return e.download(i)

    def energy(self, mol: int = 0) -> np.ndarray:
        e, i = self._at(mol)
        return e.energy(i)

    def observables(self, mol: int = 0) -> dict:
        e, i = self._at(mol)
        return e.observables(i)

    def checkpoint(self, mol: int = 0) -> bytes:
        e, i = self._at(mol)
        return e.checkpoint(i)

    def restore(self, mol: int, blob: bytes) -> None:
        e, i = self._at(mol)
        e.restore(i, blob)

    def upload_state(self, mol: int, unc_pos, pos=None, vel=None) -> None:
        e, i = self._at(mol)
        e.upload_state(i, unc_pos, pos, vel)

    def _rows(self) -> list[tuple[int, int]]:
        starts = np.cumsum([0] + [m.n for m in self.mols])
        return [(int(starts[c0]), int(starts[c1])) for c0, c1 in zip(self.cuts[:-1], self.cuts[1:])]

    def download_all(self, out: np.ndarray | None = None) -> np.ndarray:
        """Coordinates of every bead, molecules in id order, shape (total, 3)."""
        total = sum(m.n for m in self.mols)
        if out is None:
            out = np.empty((total, 3), np.float32)
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.size == 3 * total
        out2 = out.reshape(total, 3)
        for e, (r0, r1) in zip(self.engines, self._rows()):
            e.download_all(out2[r0:r1])
        return out

    def download_all_async(self, out: np.ndarray) -> list[int]:
        """Queues every context's copy into its rows of `out` (page-locked,
        alive until the wait); returns the tickets for download_wait."""
        total = sum(m.n for m in self.mols)
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.size == 3 * total
        out2 = out.reshape(total, 3)
        return [e.download_all_async(out2[r0:r1]) for e, (r0, r1) in zip(self.engines, self._rows())]

    def download_wait(self, tickets: list[int]) -> None:
        for e, t in zip(self.engines, tickets):
            e.download_wait(t)

    def list_sizes(self) -> dict:
        out: dict = {}
        for e in self.engines:
            for k, v in e.list_sizes().items():
                out[k] = out.get(k, 0) + v
        return out

    def tuning(self) -> list[dict]:
        return [e.tuning() for e in self.engines]


def _describe(mol: Molecule, xyz, T, traj, nsteps, keep: list, vel=None, eps_energy=None):
    x = np.ascontiguousarray(mol.xyz if xyz is None else xyz, np.float32)
    arrs = dict(bi=mol.bond_i, bj=mol.bond_j, br=mol.bond_r0, ai=mol.ang_i, ak=mol.ang_k,
                ni=mol.nat_i, nj=mol.nat_j, nr=mol.nat_r0, ne=mol.nat_eps, ty=mol.types)
    a = {k: np.ascontiguousarray(v, np.float32 if k in ("br", "nr", "ne") else np.int32)
         for k, v in arrs.items()}
    v = None if vel is None else np.ascontiguousarray(vel, np.float32)
    ee = None if eps_energy is None else np.ascontiguousarray(eps_energy, np.float32)
    keep += [x, v, ee, *a.values()]
    return MoleculeDesc(mol.n, len(a["bi"]), _p(a["bi"]), _p(a["bj"]), _p(a["br"]),
                        len(a["ai"]), _p(a["ai"]), _p(a["ak"]), len(a["ni"]), _p(a["ni"]),
                        _p(a["nj"]), _p(a["nr"]), _p(a["ne"]), _p(ee), _p(a["ty"]), _p(x),
                        None, _p(v), float(T), int(traj), int(nsteps))


class Server:
    """A served context (include/sop_gpu.h, sop_serve_*): jobs submitted while
    others run, admitted by HBM budget at neighbour-list boundaries."""

    def __init__(self, params: Params, budget_bytes: int, max_job_beads: int):
        self.params = params
        h = ctypes.c_void_p()
        rc = lib().sop_serve_create(ctypes.byref(params), int(budget_bytes), int(max_job_beads),
                                    ctypes.byref(h))
        if rc != SOP_OK:
            raise SopError(rc, (lib().sop_last_error(None) or b"").decode())
        self.h = h
        self.sizes = {}

    def _check(self, rc):
        if rc != SOP_OK:
            raise SopError(rc, (lib().sop_last_error(self.h) or b"").decode())

    def submit(self, mol: Molecule, xyz=None, nsteps: int = 1000, T: float = 0.6,
               traj: int = 0) -> int:
        keep = []
        d = _describe(mol, xyz, T, traj, nsteps, keep)
        job = ctypes.c_int()
        self._check(lib().sop_serve_submit(self.h, ctypes.byref(d), ctypes.byref(job)))
        self.sizes[job.value] = mol.n
        return job.value

    def advance(self, rounds: int = 1) -> None:
        self._check(lib().sop_serve_advance(self.h, int(rounds)))

    def checkpoint(self, job: int) -> bytes:
        """Exact checkpoint of a running job, between rounds (sop_serve_checkpoint)."""
        size = ctypes.c_longlong()
        self._check(lib().sop_serve_checkpoint(self.h, job, None, 0, ctypes.byref(size)))
        buf = ctypes.create_string_buffer(size.value)
        self._check(lib().sop_serve_checkpoint(self.h, job, buf, size.value, ctypes.byref(size)))
        return buf.raw[:size.value]

    def resume(self, mol: Molecule, blob: bytes, nsteps: int, T: float = 0.6, traj: int = 0) -> int:
        """Queue a job that continues from a checkpoint (sop_serve_resume);
        nsteps is the job's total step budget."""
        keep = []
        d = _describe(mol, None, T, traj, nsteps, keep)
        job = ctypes.c_int()
        self._check(lib().sop_serve_resume(self.h, ctypes.byref(d), blob, len(blob),
                                           ctypes.byref(job)))
        self.sizes[job.value] = mol.n
        return job.value

    def finished(self) -> list[int]:
        out = np.zeros(4096, np.int32)
        cnt = ctypes.c_int()
        self._check(lib().sop_serve_finished(self.h, len(out), _p(out), ctypes.byref(cnt)))
        return out[:cnt.value].tolist()

    def result(self, job: int) -> dict:
        n = self.sizes[job]
        unc = np.empty((n, 3), np.float32)
        vel = np.empty((n, 3), np.float32)
        en = np.zeros(5, np.float64)
        st, steps, lat = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_double()
        self._check(lib().sop_serve_result(self.h, job, _p(unc), _p(vel), _p(en), ctypes.byref(st),
                                           ctypes.byref(steps), ctypes.byref(lat)))
        return {"unc_pos": unc, "vel": vel, "energy": en, "status": st.value,
                "steps": steps.value, "latency_s": lat.value}

    def stats(self) -> dict:
        o = np.zeros(8, np.int64)
        self._check(lib().sop_serve_stats(self.h, _p(o)))
        keys = ("queued", "active", "finished", "active_beads", "bead_capacity", "device_bytes",
                "budget", "clock")
        return dict(zip(keys, (int(v) for v in o)))

    def run_until_idle(self, max_rounds: int = 100000) -> None:
        for _ in range(max_rounds):
            s = self.stats()
            if s["queued"] == 0 and s["active"] == 0:
                return
            self.advance(1)
        raise RuntimeError("server did not drain")

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().sop_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def plain(mol: Molecule, xyz=None, params: Params | None = None, T: float = 0.6, traj: int = 0,
          **kw) -> Engine:
    """The reference's plain path: one molecule in its own context, committed."""
    e = Engine(params)
    e.add(mol, xyz, T=T, traj=traj, **kw)
    e.commit()
    return e
