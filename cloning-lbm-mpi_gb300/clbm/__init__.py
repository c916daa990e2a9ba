"""ctypes binding of libclbm's C ABI (include/clbm.h).

This is glue for tests, the smoke entry point and the benchmark: every call
goes straight to the C ABI, there is no Python compute path.  The library is
the in-tree build ``cloning-lbm-mpi_gb300/_build/libclbm.so``; loading fails
loudly when it is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent.parent
LIB_PATH = PKG / "_build" / "libclbm.so"

OK, ERR_INVALID, ERR_CUDA, ERR_DEVICE, ERR_NOMEM, ERR_IO = 0, -1, -2, -3, -4, -5
FP64, FP32 = 0, 1
RESAMPLE_REFERENCE, RESAMPLE_SYSTEMATIC = 0, 1
PERTURB_NONE, PERTURB_MIX, PERTURB_UNIFORM = 0, 1, 2
DRAG_STRESS, DRAG_MOMENTUM = 0, 1
FLAG_GRAPH = 1
VARIANT_PER_RUN = -1

# every entry point include/clbm.h declares, for the export check
EXPORTS = [
    "clbm_strerror", "clbm_last_error", "clbm_version", "clbm_device_count",
    "clbm_ref_stream_collide", "clbm_ref_stream_collide_spatial", "clbm_ref_walls_bb",
    "clbm_ref_square_bb", "clbm_ref_interior_reset", "clbm_ref_force_on_square",
    "clbm_ref_perturbed_state", "clbm_ref_perturbed_state_noalloc", "clbm_create", "clbm_destroy", "clbm_load_pops_aos_f64",
    "clbm_load_run_aos_f64", "clbm_dump_pops_aos_f64", "clbm_set_snapshots_aos_f64",
    "clbm_init_equilibrium", "clbm_run_interval", "clbm_get_drag", "clbm_clone_step",
    "clbm_get_clone_result", "clbm_get_rvalues", "clbm_intervals_done", "clbm_scgf",
    "clbm_set_pending_labels", "clbm_macro_fields", "clbm_get_field_map", "clbm_enable_history", "clbm_reconstruct_lineages", "clbm_drag_fwd", "clbm_drag_bwd", "clbm_get_drag_grad_aos_f64", "clbm_run_sampler", "clbm_run_sampler_outputs", "clbm_profile", "clbm_profile_read", "clbm_profile_read_fields", "clbm_autotune", "clbm_set_step_variant", "clbm_set_run_variants", "clbm_get_run_variants", "clbm_band_rows", "clbm_set_band_rows", "clbm_get_band_rows", "clbm_shard_plan", "clbm_ref_random_field",
    "clbm_error_word", "clbm_sync", "clbm_stream",
]


class Geom(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nx", "ny", "xmin", "xmax", "ymin", "ymax")]


class RunDesc(C.Structure):
    _fields_ = [
        ("width", C.c_int), ("height", C.c_int),
        ("xmin", C.c_int), ("xmax", C.c_int), ("ymin", C.c_int), ("ymax", C.c_int),
        ("nclones", C.c_int), ("ranks", C.c_int),
        ("tau", C.c_double), ("beta", C.c_double), ("alpha", C.c_double),
        ("force_scale", C.c_double), ("force_shift", C.c_double), ("dt", C.c_double),
        ("perturb_mode", C.c_int), ("resample_mode", C.c_int),
        ("eps", C.c_double), ("seed", C.c_ulonglong), ("nsnap", C.c_int), ("drag_mode", C.c_int),
        ("field_mode", C.c_int), ("field_steps", C.c_int), ("field_eps", C.c_double),
        ("field_sigma", C.c_double),
    ]


class ClbmError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__(f"{where}: status {status}: {msg}")
        self.status = status


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"libclbm is not built ({LIB_PATH}); run cloning-lbm-mpi_gb300/build.py")
        L = C.CDLL(str(LIB_PATH))
        L.clbm_strerror.restype = C.c_char_p
        L.clbm_last_error.restype = C.c_char_p
        L.clbm_stream.restype = C.c_void_p
        vp, d, i = C.c_void_p, C.c_double, C.c_int
        L.clbm_ref_stream_collide.argtypes = [C.POINTER(Geom), vp, vp, vp, vp, vp, d, d, vp]
        L.clbm_ref_stream_collide_spatial.argtypes = [C.POINTER(Geom), vp, vp, vp, vp, vp, d, vp, d, d, vp]
        L.clbm_ref_walls_bb.argtypes = [C.POINTER(Geom), vp, vp, vp]
        L.clbm_ref_square_bb.argtypes = [C.POINTER(Geom), vp, vp, vp]
        L.clbm_ref_interior_reset.argtypes = [C.POINTER(Geom), vp, vp]
        L.clbm_ref_force_on_square.argtypes = [C.POINTER(Geom), vp, d, C.POINTER(d), vp]
        L.clbm_ref_perturbed_state.argtypes = [vp, vp, d, i, i, vp, vp]
        L.clbm_ref_perturbed_state_noalloc.argtypes = [vp, vp, d, i, i, vp, vp]
        L.clbm_create.argtypes = [C.POINTER(RunDesc), i, i, i, i, C.POINTER(vp)]
        L.clbm_destroy.argtypes = [vp]
        L.clbm_load_pops_aos_f64.argtypes = [vp, i, i, vp]
        L.clbm_load_run_aos_f64.argtypes = [vp, i, vp]
        L.clbm_dump_pops_aos_f64.argtypes = [vp, i, i, vp]
        L.clbm_set_snapshots_aos_f64.argtypes = [vp, i, i, vp]
        L.clbm_init_equilibrium.argtypes = [vp, i, d, d, C.c_ulonglong]
        L.clbm_run_interval.argtypes = [vp, i]
        L.clbm_get_drag.argtypes = [vp, i, vp]
        L.clbm_clone_step.argtypes = [vp]
        L.clbm_get_clone_result.argtypes = [vp, i, vp, vp, vp, vp, vp]
        L.clbm_run_sampler.argtypes = [vp, i, i, vp]
        L.clbm_run_sampler_outputs.argtypes = [vp, i, i, vp, vp, vp, vp]
        L.clbm_get_rvalues.argtypes = [vp, i, i, i, vp, vp]
        L.clbm_intervals_done.argtypes = [vp, i, C.POINTER(i)]
        L.clbm_scgf.argtypes = [vp, i, i, i, d, C.POINTER(d)]
        L.clbm_set_pending_labels.argtypes = [vp, i, vp]
        L.clbm_macro_fields.argtypes = [vp, i, i, vp, vp, vp]
        L.clbm_get_field_map.argtypes = [vp, i, i, vp, C.POINTER(i)]
        L.clbm_enable_history.argtypes = [vp, i]
        L.clbm_reconstruct_lineages.argtypes = [vp, i, C.POINTER(i), vp, vp]
        L.clbm_drag_fwd.argtypes = [vp, i, i, vp]
        L.clbm_drag_bwd.argtypes = [vp]
        L.clbm_get_drag_grad_aos_f64.argtypes = [vp, i, i, vp]
        L.clbm_profile.argtypes = [vp, i]
        L.clbm_autotune.argtypes = [vp, i, C.POINTER(i), vp, C.POINTER(i)]
        L.clbm_set_step_variant.argtypes = [vp, i]
        L.clbm_set_run_variants.argtypes = [vp, vp]
        L.clbm_get_run_variants.argtypes = [vp, vp]
        L.clbm_band_rows.argtypes = [C.POINTER(RunDesc), i, d, vp]
        L.clbm_set_band_rows.argtypes = [vp, i, vp, i]
        L.clbm_get_band_rows.argtypes = [vp, i, vp, C.POINTER(i)]
        L.clbm_profile_read.argtypes = [vp, C.POINTER(d), C.POINTER(i)]
        L.clbm_profile_read_fields.argtypes = [vp, C.POINTER(d), C.POINTER(i)]
        L.clbm_error_word.argtypes = [vp, C.POINTER(C.c_uint), i]
        L.clbm_sync.argtypes = [vp]
        L.clbm_stream.argtypes = [vp]
        L.clbm_shard_plan.argtypes = [vp, i, i, i, vp, C.POINTER(i), vp, C.POINTER(i), vp, C.POINTER(i)]
        L.clbm_ref_random_field.argtypes = [i, i, d, C.c_ulonglong, i, vp, C.POINTER(i)]
        _lib = L
    return _lib


def check(status: int, where: str) -> None:
    if status != OK:
        msg = lib().clbm_last_error().decode(errors="replace")
        raise ClbmError(status, where, msg or lib().clbm_strerror(status).decode())


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def device_count() -> int:
    return int(lib().clbm_device_count())


def geom(nx, ny, xmin, xmax, ymin, ymax) -> Geom:
    return Geom(nx, ny, xmin, xmax, ymin, ymax)


# ---- function level (device pointers as ints, e.g. torch .data_ptr()) ----
def ref_stream_collide(g, fin, fout, rho, ux, uy, beta, tau, stream=None):
    check(lib().clbm_ref_stream_collide(C.byref(g), fin, fout, rho, ux, uy, beta, tau, stream),
          "clbm_ref_stream_collide")


def ref_stream_collide_spatial(g, fin, fout, rho, ux, uy, beta0, map_, tau, eps, stream=None):
    check(lib().clbm_ref_stream_collide_spatial(C.byref(g), fin, fout, rho, ux, uy, beta0, map_,
                                                tau, eps, stream), "clbm_ref_stream_collide_spatial")


def ref_walls_bb(g, fout, fin, stream=None):
    check(lib().clbm_ref_walls_bb(C.byref(g), fout, fin, stream), "clbm_ref_walls_bb")


def ref_square_bb(g, fout, fin, stream=None):
    check(lib().clbm_ref_square_bb(C.byref(g), fout, fin, stream), "clbm_ref_square_bb")


def ref_interior_reset(g, fout, stream=None):
    check(lib().clbm_ref_interior_reset(C.byref(g), fout, stream), "clbm_ref_interior_reset")


def ref_force_on_square(g, f, omega, stream=None) -> float:
    out = C.c_double()
    check(lib().clbm_ref_force_on_square(C.byref(g), f, omega, C.byref(out), stream),
          "clbm_ref_force_on_square")
    return out.value


def ref_perturbed_state(fin, snaps, eps, nsnap, n, prefactors: np.ndarray, stream=None):
    pre = np.ascontiguousarray(prefactors, dtype=np.float64)
    check(lib().clbm_ref_perturbed_state(fin, snaps, eps, nsnap, n, _p(pre), stream),
          "clbm_ref_perturbed_state")


def ref_perturbed_state_noalloc(fin, snaps, eps, nsnap, n, prefactors: np.ndarray, stream=None):
    pre = np.ascontiguousarray(prefactors, dtype=np.float64)
    check(lib().clbm_ref_perturbed_state_noalloc(fin, snaps, eps, nsnap, n, _p(pre), stream),
          "clbm_ref_perturbed_state_noalloc")


# ---- sampler level ----
def ref_random_field(dx: int, dy: int, sigma: float, seed: int, draw: int) -> tuple[np.ndarray, int]:
    """clbm_ref_random_field: (map in the reference order y + dy*x, number of
    clamped negative eigenvalues)."""
    out = np.empty(dx * dy)
    neg = C.c_int()
    check(lib().clbm_ref_random_field(dx, dy, sigma, seed, draw, _p(out), C.byref(neg)), "clbm_ref_random_field")
    return out, neg.value


def shard_plan(labels: np.ndarray, nshards: int, shard: int) -> dict:
    """clbm_shard_plan: this shard's sends, receives and local copies, each an
    (n, 3) int array of (src_slot, dst_slot, peer) in ascending dst_slot."""
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    n = lab.size
    out = {k: np.zeros((n, 3), dtype=np.int32) for k in ("sends", "recvs", "locals")}
    cnt = {k: C.c_int() for k in out}
    check(lib().clbm_shard_plan(_p(lab), n, nshards, shard, _p(out["sends"]), C.byref(cnt["sends"]),
                                _p(out["recvs"]), C.byref(cnt["recvs"]), _p(out["locals"]),
                                C.byref(cnt["locals"])), "clbm_shard_plan")
    return {k: out[k][:cnt[k].value] for k in out}


# Interval-kernel variant numbering of clbm_autotune / clbm_set_step_variant:
# 0..7 the streaming step kernel's launch variants (one launch per step), then
# the cluster-resident interval kernel for cluster sizes 1, 2, 4, 8, 16 times
# thread counts 1024, 512, 256 (one launch per run per interval).
STREAM_VARIANTS = 8
TEMPORAL_THREADS = (1024, 512, 256)
CLUSTER_SIZES = (1, 2, 4, 8, 16, 3, 5, 6, 7, 9, 10)  # the autotuner's numbering order


def band_rows(run: RunDesc, cluster_size: int, gamma: float) -> np.ndarray:
    """The band split of a lattice over a cluster balanced for weight gamma
    (host-only: no device needed)."""
    a = np.zeros(cluster_size, np.int32)
    check(lib().clbm_band_rows(C.byref(run), cluster_size, gamma, _p(a)), "clbm_band_rows")
    return a


def describe_variant(v: int) -> dict:
    if v < STREAM_VARIANTS:
        return {"kind": "streaming", "kernel": "k_step_f32", "variant": v}
    q = v - STREAM_VARIANTS
    return {"kind": "cluster-resident", "kernel": "k_temporal_f32", "variant": v,
            "cluster_size": CLUSTER_SIZES[q // len(TEMPORAL_THREADS)],
            "threads": TEMPORAL_THREADS[q % len(TEMPORAL_THREADS)]}


class Sampler:
    """One clbm context: every clone of one or several runs on the device."""

    def __init__(self, runs: list[RunDesc], precision: int = FP64, max_steps: int = 1000,
                 flags: int = 0):
        arr = (RunDesc * len(runs))(*runs)
        h = C.c_void_p()
        check(lib().clbm_create(arr, len(runs), precision, max_steps, flags, C.byref(h)), "clbm_create")
        self.h = h
        self.runs = list(runs)
        self.precision = precision
        self.last_steps = 0

    def close(self):
        if self.h:
            lib().clbm_destroy(self.h)
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

    def n(self, run=0) -> int:
        r = self.runs[run]
        return 9 * r.width * r.height

    def load_run(self, run: int, aos: np.ndarray):
        a = np.ascontiguousarray(aos, dtype=np.float64)
        assert a.size == self.runs[run].nclones * self.n(run)
        check(lib().clbm_load_run_aos_f64(self.h, run, _p(a)), "clbm_load_run_aos_f64")

    def load(self, run: int, clone: int, aos: np.ndarray):
        a = np.ascontiguousarray(aos, dtype=np.float64)
        assert a.size == self.n(run)
        check(lib().clbm_load_pops_aos_f64(self.h, run, clone, _p(a)), "clbm_load_pops_aos_f64")

    def dump(self, run: int, clone: int) -> np.ndarray:
        out = np.empty(self.n(run))
        check(lib().clbm_dump_pops_aos_f64(self.h, run, clone, _p(out)), "clbm_dump_pops_aos_f64")
        return out

    def set_snapshots(self, run: int, snaps: np.ndarray):
        a = np.ascontiguousarray(snaps, dtype=np.float64)
        nsnap = a.size // self.n(run)
        check(lib().clbm_set_snapshots_aos_f64(self.h, run, nsnap, _p(a)), "clbm_set_snapshots_aos_f64")

    def init_equilibrium(self, run: int, u0: float, noise: float, seed: int):
        check(lib().clbm_init_equilibrium(self.h, run, u0, noise, seed), "clbm_init_equilibrium")

    def run_interval(self, steps: int):
        check(lib().clbm_run_interval(self.h, steps), "clbm_run_interval")
        self.last_steps = steps

    def drag(self, run: int = 0) -> np.ndarray:
        out = np.empty((self.runs[run].nclones, self.last_steps))
        check(lib().clbm_get_drag(self.h, run, _p(out)), "clbm_get_drag")
        return out

    def clone_step(self):
        check(lib().clbm_clone_step(self.h), "clbm_clone_step")

    def clone_result(self, run: int = 0) -> dict:
        nc = self.runs[run].nclones
        labels = np.empty(nc, np.int32)
        w = np.empty(nc)
        pre = np.empty(nc, np.int32)
        post = np.empty(nc, np.int32)
        rv = C.c_double()
        check(lib().clbm_get_clone_result(self.h, run, _p(labels), C.byref(rv), _p(w), _p(pre), _p(post)),
              "clbm_get_clone_result")
        return {"labels": labels, "rvalue": rv.value, "weights": w, "copies_pre": pre, "copies_post": post}

    def intervals_done(self, run: int = 0) -> int:
        n = C.c_int()
        check(lib().clbm_intervals_done(self.h, run, C.byref(n)), "clbm_intervals_done")
        return n.value

    def rvalues(self, run: int = 0, first: int = 0, count: int | None = None):
        if count is None:
            count = self.intervals_done(run) - first
        rv, lr = np.empty(count), np.empty(count)
        check(lib().clbm_get_rvalues(self.h, run, first, count, _p(rv), _p(lr)), "clbm_get_rvalues")
        return rv, lr

    def scgf(self, run: int, dT: float, first: int = 0, count: int | None = None) -> float:
        if count is None:
            count = self.intervals_done(run) - first
        out = C.c_double()
        check(lib().clbm_scgf(self.h, run, first, count, dT, C.byref(out)), "clbm_scgf")
        return out.value

    def macro(self, run: int, clone: int):
        n = self.runs[run].width * self.runs[run].height
        rho, ux, uy = np.empty(n), np.empty(n), np.empty(n)
        check(lib().clbm_macro_fields(self.h, run, clone, _p(rho), _p(ux), _p(uy)), "clbm_macro_fields")
        return rho, ux, uy

    def field_map(self, run: int, clone: int):
        """(map in the reference order y + H*x, clamped negative eigenvalues)"""
        r = self.runs[run]
        out = np.empty(r.width * r.height)
        neg = C.c_int()
        check(lib().clbm_get_field_map(self.h, run, clone, _p(out), C.byref(neg)), "clbm_get_field_map")
        return out, neg.value

    def enable_history(self, max_intervals: int):
        check(lib().clbm_enable_history(self.h, max_intervals), "clbm_enable_history")

    def reconstruct(self, run: int, steps: int):
        """(lineage drag series [nclones][n*steps], ancestors [nclones][n])"""
        n = C.c_int()
        check(lib().clbm_reconstruct_lineages(self.h, run, C.byref(n), None, None), "clbm_reconstruct_lineages")
        nc = self.runs[run].nclones
        out = np.empty((nc, n.value * steps))
        anc = np.empty((nc, n.value), np.int32)
        check(lib().clbm_reconstruct_lineages(self.h, run, C.byref(n), _p(out), _p(anc)),
              "clbm_reconstruct_lineages")
        return out, anc

    def drag_fwd(self, steps: int, every: int) -> np.ndarray:
        J = np.empty(sum(r.nclones for r in self.runs))
        check(lib().clbm_drag_fwd(self.h, steps, every, _p(J)), "clbm_drag_fwd")
        self.last_steps = steps
        return J

    def drag_bwd(self):
        check(lib().clbm_drag_bwd(self.h), "clbm_drag_bwd")

    def drag_grad(self, run: int, clone: int) -> np.ndarray:
        out = np.empty(self.n(run))
        check(lib().clbm_get_drag_grad_aos_f64(self.h, run, clone, _p(out)), "clbm_get_drag_grad_aos_f64")
        return out

    def set_pending_labels(self, run: int, labels: np.ndarray):
        a = np.ascontiguousarray(labels, dtype=np.int32)
        check(lib().clbm_set_pending_labels(self.h, run, _p(a)), "clbm_set_pending_labels")

    def run_sampler(self, steps: int, intervals: int) -> np.ndarray:
        rv = np.empty((len(self.runs), intervals))
        check(lib().clbm_run_sampler(self.h, steps, intervals, _p(rv)), "clbm_run_sampler")
        self.last_steps = steps
        return rv

    def run_sampler_outputs(self, steps: int, intervals: int, out: dict | None = None) -> dict:
        """clbm_run_sampler_outputs: R_t, and every interval's drag series
        [interval][clone][step], labels and weights [interval][clone] (all
        runs' clones in run order).  `out` may hold preallocated arrays."""
        n = sum(r.nclones for r in self.runs)
        out = out if out is not None else {}
        rv = out.setdefault("rvalues", np.empty((len(self.runs), intervals)))
        drag = out.setdefault("drag", np.empty((intervals, n, steps)))
        labels = out.setdefault("labels", np.empty((intervals, n), np.int32))
        weights = out.setdefault("weights", np.empty((intervals, n)))
        check(lib().clbm_run_sampler_outputs(self.h, steps, intervals, _p(rv), _p(drag), _p(labels), _p(weights)),
              "clbm_run_sampler_outputs")
        self.last_steps = steps
        return out

    def autotune(self, launches: int = 5, measure: bool = True):
        """Returns (best variant, ms per launch of every variant)."""
        best, nv = C.c_int(), C.c_int()
        ms = np.zeros(64)
        check(lib().clbm_autotune(self.h, launches, C.byref(best), _p(ms) if measure else None,
                                  C.byref(nv)), "clbm_autotune")
        return best.value, ms[:nv.value]

    def set_step_variant(self, v: int):
        check(lib().clbm_set_step_variant(self.h, v), "clbm_set_step_variant")

    def set_run_variants(self, variants):
        a = np.ascontiguousarray(variants, dtype=np.int32)
        check(lib().clbm_set_run_variants(self.h, _p(a)), "clbm_set_run_variants")

    def run_variants(self) -> np.ndarray:
        a = np.zeros(len(self.runs), np.int32)
        check(lib().clbm_get_run_variants(self.h, _p(a)), "clbm_get_run_variants")
        return a

    def set_band_rows(self, run: int, rows):
        a = np.ascontiguousarray(rows, dtype=np.int32)
        check(lib().clbm_set_band_rows(self.h, run, _p(a) if a.size else None, int(a.size)),
              "clbm_set_band_rows")

    def band_rows(self, run: int) -> np.ndarray:
        a = np.zeros(16, np.int32)
        n = C.c_int()
        check(lib().clbm_get_band_rows(self.h, run, _p(a), C.byref(n)), "clbm_get_band_rows")
        return a[:n.value].copy()

    def profile(self, enable: bool):
        check(lib().clbm_profile(self.h, int(enable)), "clbm_profile")

    def profile_read(self) -> tuple[float, int]:
        ms, n = C.c_double(), C.c_int()
        check(lib().clbm_profile_read(self.h, C.byref(ms), C.byref(n)), "clbm_profile_read")
        return ms.value, n.value

    def profile_read_fields(self) -> tuple[float, int]:
        ms, n = C.c_double(), C.c_int()
        check(lib().clbm_profile_read_fields(self.h, C.byref(ms), C.byref(n)), "clbm_profile_read_fields")
        return ms.value, n.value

    def error_word(self, clear: bool = False) -> int:
        w = C.c_uint()
        check(lib().clbm_error_word(self.h, C.byref(w), int(clear)), "clbm_error_word")
        return w.value

    def sync(self):
        check(lib().clbm_sync(self.h), "clbm_sync")

    def stream(self) -> int:
        return lib().clbm_stream(self.h) or 0
