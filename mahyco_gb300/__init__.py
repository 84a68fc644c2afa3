"""GB300-native implementation of MaHyCo's per-cycle hydro hot path.

Python mirror of the reference's entry points, bound to the C ABI of
include/hydro_gb300.h (libmahyco_gb300.so, built in-tree by
mahyco_gb300.build):

  parse_deck(path)          LectureDonnees (lecture_donnees/LectureDonnees.cc)
  Run(spec).simulate()      Vnr::simulate (vnr_remap/VnrRemap.cc:289-346)
  Run.step(n)               cycles of Vnr::executeTimeLoopN (VnrRemap.cc:127)
  Run.fetch(name)           the arrays dumpVariables writes (VnrRemap.cc:255)

There is no CPU fallback: every call runs the CUDA kernels, and importing
this module without the built library, or calling it without a GPU, raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libmahyco_gb300.so"

SCHEME_EUCCLHYD = 2000
SCHEME_VNR = 2001
LIMITERS = {"minmod": 300, "superBee": 301, "vanLeer": 302, "minmodG": 1300,
            "superBeeG": 1301, "vanLeerG": 1302, "arithmeticG": 1303,
            "ultrabeeG": 1304}
ERR_NAN, ERR_ENERGY, ERR_DT_MIN, ERR_NEGATIVE = 1, 2, 4, 8


class HydroSpec(C.Structure):
    """ctypes mirror of struct hydro_spec (include/hydro_gb300.h)."""

    _fields_ = [
        ("scheme", C.c_int), ("test_case", C.c_int), ("nx", C.c_int),
        ("ny", C.c_int), ("dx", C.c_double), ("dy", C.c_double),
        ("nbmat", C.c_int), ("eos", C.c_int * 3), ("gamma", C.c_double * 3),
        ("gamma_scalar", C.c_double), ("final_time", C.c_double),
        ("output_time", C.c_double), ("dt_init", C.c_double),
        ("dt_min", C.c_double), ("cfl", C.c_double), ("max_cycles", C.c_long),
        ("space_order", C.c_int), ("projection", C.c_int),
        ("projection_conservative", C.c_int), ("projection_order", C.c_int),
        ("threshold", C.c_double), ("limiter", C.c_int), ("pb", C.c_int),
        ("pb_mixte", C.c_int), ("limiter_pure", C.c_int),
        ("pb_complet", C.c_int), ("pseudo_centree", C.c_int),
        ("dual_mass_flux", C.c_int), ("sans_lagrange", C.c_int),
        ("init_variant", C.c_int), ("energy_limit", C.c_double),
    ]

    def copy(self) -> "HydroSpec":
        s = HydroSpec()
        C.pointer(s)[0] = self
        return s

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            val = getattr(self, name)
            out[name] = list(val) if hasattr(val, "__len__") else val
        return out


class ServeDone(C.Structure):
    """struct hydro_serve_done"""
    _fields_ = [("req_id", C.c_long), ("status", C.c_int), ("latency_s", C.c_double),
                ("cycles", C.c_long), ("cells", C.c_long), ("wait_s", C.c_double),
                ("resident_s", C.c_double)]


class ServeStats(C.Structure):
    """struct hydro_serve_stats"""
    _fields_ = [("submitted", C.c_long), ("admitted", C.c_long), ("completed", C.c_long),
                ("failed", C.c_long), ("resident", C.c_long), ("waiting", C.c_long),
                ("peak_resident", C.c_long), ("ticks", C.c_long), ("cycles", C.c_long),
                ("bytes_in_use", C.c_size_t), ("peak_bytes", C.c_size_t),
                ("cell_updates", C.c_double), ("busy_s", C.c_double)]


_lib = None


def lib() -> C.CDLL:
    """Loads libmahyco_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: run `python -m mahyco_gb300.build` "
                "(the CUDA path has no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        vp, i, sz = C.c_void_p, C.c_int, C.c_size_t
        L.hydro_last_error.restype = C.c_char_p
        L.hydro_spec_default.argtypes = [C.POINTER(HydroSpec)]
        L.hydro_spec_parse_deck.argtypes = [C.c_char_p, C.POINTER(HydroSpec)]
        L.hydro_ctx_create.argtypes = [i, sz, C.POINTER(vp)]
        L.hydro_ctx_destroy.argtypes = [vp]
        L.hydro_ctx_destroy.restype = None
        L.hydro_ctx_stream.argtypes = [vp]
        L.hydro_ctx_stream.restype = vp
        L.hydro_run_create.argtypes = [vp, C.POINTER(HydroSpec), C.POINTER(vp)]
        L.hydro_run_step.argtypes = [vp, i, C.POINTER(i)]
        L.hydro_run_enqueue.argtypes = [vp, i]
        L.hydro_run_checkpoint.argtypes = [vp, C.c_char_p]
        L.hydro_run_restore.argtypes = [vp, C.c_char_p, C.POINTER(vp)]
        L.hydro_run_step_to_output.argtypes = [vp, i, C.c_double, C.POINTER(i),
                                               C.POINTER(i)]
        L.hydro_run_sync.argtypes = [vp, C.POINTER(i)]
        L.hydro_run_fetch.argtypes = [vp, C.c_char_p, C.POINTER(C.c_double), sz]
        L.hydro_run_field_size.argtypes = [vp, C.c_char_p]
        L.hydro_run_field_size.restype = sz
        L.hydro_run_time.argtypes = [vp, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), C.POINTER(C.c_long)]
        L.hydro_run_error.argtypes = [vp, C.POINTER(C.c_uint), C.POINTER(C.c_long)]
        L.hydro_run_destroy.argtypes = [vp]
        L.hydro_run_kernel_launches.argtypes = [vp]
        L.hydro_run_kernel_launches.restype = C.c_longlong
        L.hydro_run_device_bytes.argtypes = [vp]
        L.hydro_run_device_bytes.restype = sz
        L.hydro_run_timed.argtypes = [vp, i, C.POINTER(C.c_float)]
        L.hydro_run_profile.argtypes = [vp, i, C.POINTER(C.c_double),
                                        C.POINTER(C.c_longlong), i]
        L.hydro_kernel_name.argtypes = [i]
        L.hydro_kernel_name.restype = C.c_char_p
        L.hydro_kernel_kinds.restype = i
        L.hydro_fp64_peak.argtypes = [i, C.POINTER(C.c_double)]
        L.hydro_softfp_check.argtypes = [i, vp, vp, vp, vp, vp, C.c_longlong, vp]
        L.hydro_softfp_rates.argtypes = [i, C.POINTER(C.c_double)]
        runs_t = C.POINTER(vp)
        L.hydro_batch_step.argtypes = [vp, runs_t, i, i, C.POINTER(i)]
        L.hydro_batch_enqueue.argtypes = [vp, runs_t, i, i]
        L.hydro_batch_timed.argtypes = [vp, runs_t, i, i, C.POINTER(C.c_float)]
        L.hydro_batch_profile.argtypes = [vp, runs_t, i, i, C.POINTER(C.c_double),
                                          C.POINTER(C.c_longlong), i]
        L.hydro_batch_config.argtypes = [vp, C.POINTER(i), C.POINTER(i), C.POINTER(i), i]
        L.hydro_batch_set_tuning.argtypes = [vp, i]
        L.hydro_batch_kernel_launches.argtypes = [vp]
        L.hydro_batch_kernel_launches.restype = C.c_longlong
        L.hydro_serve_config.argtypes = [vp, sz, i, i, i]
        L.hydro_serve_submit.argtypes = [vp, C.POINTER(HydroSpec), i, C.POINTER(C.c_long)]
        L.hydro_serve_poll.argtypes = [vp, C.c_double, C.POINTER(ServeDone)]
        L.hydro_serve_result.argtypes = [vp, C.c_long]
        L.hydro_serve_result.restype = vp
        L.hydro_serve_release.argtypes = [vp, C.c_long]
        L.hydro_serve_stats_get.argtypes = [vp, C.POINTER(ServeStats)]
        L.hydro_serve_stop.argtypes = [vp, i]
        _lib = L
    return _lib


def _check(rc: int, what: str) -> None:
    if rc != 0:
        msg = lib().hydro_last_error().decode(errors="replace")
        raise RuntimeError(f"{what} failed ({rc}): {msg}")


def fp64_peak_tflops(device: int = 0) -> float:
    """Measured FP64 FMA throughput of the device (TFLOP/s)."""
    t = C.c_double()
    _check(lib().hydro_fp64_peak(device, C.byref(t)), "hydro_fp64_peak")
    return t.value


def softfp_rates(device: int = 0) -> dict:
    """Operations per second of dependent FP64 chains: the FP64 instruction
    against the integer-pipe form, for mul, add, div and sqrt."""
    r = (C.c_double * 8)()
    _check(lib().hydro_softfp_rates(device, r), "hydro_softfp_rates")
    return {op: {"fp64_pipe": r[2 * k], "integer_pipe": r[2 * k + 1]}
            for k, op in enumerate(("mul", "add", "div", "sqrt"))}


def default_spec() -> HydroSpec:
    s = HydroSpec()
    _check(lib().hydro_spec_default(C.byref(s)), "hydro_spec_default")
    return s


def parse_deck(path: str | os.PathLike) -> HydroSpec:
    """Reads a MaHyCo input deck (donnees.txt) into a HydroSpec."""
    s = HydroSpec()
    _check(lib().hydro_spec_parse_deck(str(path).encode(), C.byref(s)),
           "hydro_spec_parse_deck")
    return s


_CASE_NAMES = {0: "UnitTestCase", 1: "SedovTestCase", 2: "TriplePoint",
               4: "SodCaseX", 5: "SodCaseY", 6: "NohTestCase", 7: "AdvectionX",
               8: "AdvectionY", 9: "AdvectionVitX", 10: "AdvectionVitY",
               11: "BiUnitTestCase", 12: "BiSedovTestCase", 13: "BiTriplePoint",
               14: "BiShockBubble", 15: "BiSodCaseX", 16: "BiSodCaseY",
               17: "BiNohTestCase", 18: "BiAdvectionX", 19: "BiAdvectionY",
               20: "BiAdvectionVitX", 21: "BiAdvectionVitY"}


def deck_text(spec: HydroSpec) -> str:
    """The positional deck (key order of lecture_donnees/LectureDonnees.cc)
    that parse_deck reads back into the same options: test case, mesh, times,
    one EOS per material, scheme, orders, projection and limiter keys.  Only
    what the deck format carries is written (no cycle cap, exponents, CFL or
    init variant)."""
    lim_name = {v: k for k, v in LIMITERS.items()}
    on = lambda b: "oui" if b else "non"  # noqa: E731
    lines = ["# Cas test", _CASE_NAMES[spec.test_case],
             "# Nombre de Mailles en X", str(spec.nx),
             "# Nombre de Mailles en Y", str(spec.ny),
             "# DELTA_X", repr(spec.dx), "# DELTA_Y", repr(spec.dy),
             "# temps final", repr(spec.final_time),
             "# Temps entre deux sorties", repr(spec.output_time),
             "# Pas de temps initial", repr(spec.dt_init),
             "# Pas de temps minimal", repr(spec.dt_min)]
    for m in range(spec.nbmat):
        lines += ["# equation d'etat", "PerfectGas" if spec.eos[m] == 101 else "Void"]
    lines += ["# schema Lagrange", "VNR" if spec.scheme == SCHEME_VNR else "Eucclhyd",
              "# ordre en espace", str(spec.space_order),
              "# avec projection", on(spec.projection),
              "# projection conservative", on(spec.projection_conservative),
              "# Limite fraction volumique", repr(spec.threshold),
              "# Ordre de la projection", str(spec.projection_order),
              "# Limiteurs", lim_name[spec.limiter],
              "# option Pente Borne", on(spec.pb)]
    if spec.pb:
        lines += ["# Pente Borne mixte", on(spec.pb_mixte),
                  "# limiteur mailles pures", lim_name.get(spec.limiter_pure, "minmod"),
                  "# Pente Borne complet", on(spec.pb_complet)]
    if spec.scheme == SCHEME_VNR:
        lines += ["# pseudo_centree", on(spec.pseudo_centree)]
        if spec.projection:
            lines += ["# methode flux masse", ["A1", "A2", "PB"][spec.dual_mass_flux]]
    return "\n".join(lines) + "\n"


def write_deck(spec: HydroSpec, path: str | os.PathLike) -> None:
    with open(path, "w") as f:
        f.write(deck_text(spec))


def driver_path() -> str:
    """The drop-in command-line driver (mahyco_gb300_run <deck>)."""
    from . import build as _b
    return str(_b.OUT / "mahyco_gb300_run")


class Context:
    """One GPU, one CUDA stream, an optional HBM budget."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self.h = C.c_void_p()
        _check(lib().hydro_ctx_create(device, hbm_budget, C.byref(self.h)),
               "hydro_ctx_create")

    def close(self):
        if self.h:
            lib().hydro_ctx_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return lib().hydro_ctx_stream(self.h) or 0


_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class Run:
    """One hydro run resident in HBM (a Vnr scheme instance)."""

    def __init__(self, spec: HydroSpec, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.spec = spec
        self.owner = True
        self.h = C.c_void_p()
        _check(lib().hydro_run_create(self.ctx.h, C.byref(spec), C.byref(self.h)),
               "hydro_run_create")

    @classmethod
    def borrowed(cls, handle: int, spec: HydroSpec, ctx: Context) -> "Run":
        """A view of a run owned by someone else (e.g. the serving loop)."""
        r = cls.__new__(cls)
        r.ctx, r.spec, r.owner = ctx, spec, False
        r.h = C.c_void_p(handle)
        return r

    def close(self):
        if self.h and self.owner:
            lib().hydro_run_destroy(self.h)
        self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, ncycles: int = 1) -> bool:
        """Runs up to ncycles cycles; returns True once the run has ended."""
        done = C.c_int(0)
        _check(lib().hydro_run_step(self.h, ncycles, C.byref(done)), "hydro_run_step")
        return bool(done.value)

    def checkpoint(self, path: str | os.PathLike) -> None:
        """Writes the run's options and device state to path (between
        cycles); Run.restore continues it bit for bit."""
        _check(lib().hydro_run_checkpoint(self.h, os.fspath(path).encode()),
               "hydro_run_checkpoint")

    @classmethod
    def restore(cls, path: str | os.PathLike, ctx: "Context | None" = None) -> "Run":
        ctx = ctx or default_context()
        h = C.c_void_p()
        _check(lib().hydro_run_restore(ctx.h, os.fspath(path).encode(), C.byref(h)),
               "hydro_run_restore")
        with open(path, "rb") as f:  # the options follow the 64-byte header
            f.seek(64)
            spec = HydroSpec.from_buffer_copy(f.read(C.sizeof(HydroSpec)))
        r = cls.borrowed(h.value, spec, ctx)
        r.owner = True
        return r

    def step_to_output(self, ncycles: int, t_out: float):
        """Runs at least one and up to ncycles cycles, stopping before a
        cycle whose start time t satisfies t >= t_out or t == 0 (the
        reference's dump condition).  Returns (done, paused)."""
        done, paused = C.c_int(0), C.c_int(0)
        _check(lib().hydro_run_step_to_output(self.h, ncycles, t_out, C.byref(done),
                                              C.byref(paused)),
               "hydro_run_step_to_output")
        return bool(done.value), bool(paused.value)

    def enqueue(self, ncycles: int) -> None:
        _check(lib().hydro_run_enqueue(self.h, ncycles), "hydro_run_enqueue")

    def sync(self) -> bool:
        done = C.c_int(0)
        _check(lib().hydro_run_sync(self.h, C.byref(done)), "hydro_run_sync")
        return bool(done.value)

    def simulate(self, chunk: int = 64) -> None:
        """Runs to the end (final time or cycle cap)."""
        while not self.step(chunk):
            pass

    def fetch(self, name: str) -> np.ndarray:
        n = lib().hydro_run_field_size(self.h, name.encode())
        if n == 0:
            raise KeyError(name)
        out = np.empty(n, dtype=np.float64)
        _check(lib().hydro_run_fetch(self.h, name.encode(),
                                     out.ctypes.data_as(C.POINTER(C.c_double)), n),
               "hydro_run_fetch")
        return out

    def time(self):
        t, dt, n = C.c_double(), C.c_double(), C.c_long()
        _check(lib().hydro_run_time(self.h, C.byref(t), C.byref(dt), C.byref(n)),
               "hydro_run_time")
        return t.value, dt.value, n.value

    def error(self):
        code, cell = C.c_uint(), C.c_long()
        _check(lib().hydro_run_error(self.h, C.byref(code), C.byref(cell)),
               "hydro_run_error")
        return code.value, cell.value

    def timed(self, ncycles: int) -> float:
        """Device time (ms, CUDA events on the run's stream) of ncycles."""
        ms = C.c_float()
        _check(lib().hydro_run_timed(self.h, ncycles, C.byref(ms)), "hydro_run_timed")
        return ms.value

    def profile(self, ncycles: int) -> dict:
        """Per-kernel device time over ncycles launched one by one."""
        nk = lib().hydro_kernel_kinds()
        ms = (C.c_double * nk)()
        cnt = (C.c_longlong * nk)()
        _check(lib().hydro_run_profile(self.h, ncycles, ms, cnt, nk), "hydro_run_profile")
        return {lib().hydro_kernel_name(k).decode(): (ms[k], cnt[k]) for k in range(nk)}

    @property
    def kernel_launches(self) -> int:
        return int(lib().hydro_run_kernel_launches(self.h))

    @property
    def device_bytes(self) -> int:
        return int(lib().hydro_run_device_bytes(self.h))


BATCH_PHASES = ("lag_nodes", "lag_cells", "face_grad", "sweep_grad",
                "sweep_face", "sweep_update", "dual_grad", "dual_update",
                "final", "euc_cell_pre", "euc_nodes", "euc_cells", "euc_final")


class Batch:
    """Many runs of one context advanced together, one persistent launch per
    phase for all of them (hydro_batch_step)."""

    def __init__(self, runs: list[Run], ctx: Context | None = None):
        self.ctx = ctx or runs[0].ctx
        self.runs = list(runs)
        self._arr = (C.c_void_p * len(self.runs))(*[r.h.value for r in self.runs])

    @property
    def cells(self) -> int:
        return sum(r.spec.nx * r.spec.ny for r in self.runs)

    def step(self, ncycles: int = 1) -> int:
        """Advances every run by up to ncycles; returns the runs still going."""
        act = C.c_int(0)
        _check(lib().hydro_batch_step(self.ctx.h, self._arr, len(self.runs), ncycles,
                                      C.byref(act)), "hydro_batch_step")
        return act.value

    def enqueue(self, ncycles: int) -> None:
        _check(lib().hydro_batch_enqueue(self.ctx.h, self._arr, len(self.runs), ncycles),
               "hydro_batch_enqueue")

    def timed(self, ncycles: int) -> float:
        ms = C.c_float()
        _check(lib().hydro_batch_timed(self.ctx.h, self._arr, len(self.runs), ncycles,
                                       C.byref(ms)), "hydro_batch_timed")
        return ms.value

    def profile(self, ncycles: int) -> dict:
        nk = lib().hydro_kernel_kinds()
        ms = (C.c_double * nk)()
        cnt = (C.c_longlong * nk)()
        _check(lib().hydro_batch_profile(self.ctx.h, self._arr, len(self.runs), ncycles,
                                         ms, cnt, nk), "hydro_batch_profile")
        return {lib().hydro_kernel_name(k).decode(): (ms[k], cnt[k]) for k in range(nk)}

    def config(self) -> dict:
        n = len(BATCH_PHASES)
        w, h, g = (C.c_int * n)(), (C.c_int * n)(), (C.c_int * n)()
        rc = lib().hydro_batch_config(self.ctx.h, w, h, g, n)
        if rc < 0:
            _check(rc, "hydro_batch_config")
        return {"tuned": bool(rc),
                "phases": {BATCH_PHASES[k]: {"tile": [w[k], h[k]], "grid": g[k]}
                           for k in range(n)}}

    @property
    def kernel_launches(self) -> int:
        return int(lib().hydro_batch_kernel_launches(self.ctx.h))


def set_batch_tuning(ctx: Context, enable: bool) -> None:
    _check(lib().hydro_batch_set_tuning(ctx.h, int(enable)), "hydro_batch_set_tuning")


class Server:
    """Continuous batching of hydro runs on one context (hydro_serve_*):
    submit() returns at once; a worker thread admits requests against the
    HBM budget, advances all resident runs in batched ticks and retires each
    at its end; poll() returns completions with their latency."""

    def __init__(self, ctx: Context | None = None, budget: int = 0, max_resident: int = 0,
                 tick_cycles: int = 0, prep_threads: int = 0):
        self.ctx = ctx or default_context()
        self.specs: dict[int, HydroSpec] = {}
        _check(lib().hydro_serve_config(self.ctx.h, budget, max_resident, tick_cycles,
                                        prep_threads), "hydro_serve_config")

    def submit(self, spec: HydroSpec, keep: bool = False) -> int:
        rid = C.c_long()
        _check(lib().hydro_serve_submit(self.ctx.h, C.byref(spec), int(keep), C.byref(rid)),
               "hydro_serve_submit")
        if keep:
            self.specs[rid.value] = spec.copy()
        return rid.value

    def poll(self, timeout: float = 0.0) -> ServeDone | None:
        d = ServeDone()
        rc = lib().hydro_serve_poll(self.ctx.h, timeout, C.byref(d))
        if rc < 0:
            _check(rc, "hydro_serve_poll")
        return d if rc == 1 else None

    def result(self, req_id: int) -> Run:
        h = lib().hydro_serve_result(self.ctx.h, req_id)
        if not h:
            raise KeyError(req_id)
        return Run.borrowed(h, self.specs[req_id], self.ctx)

    def release(self, req_id: int) -> None:
        _check(lib().hydro_serve_release(self.ctx.h, req_id), "hydro_serve_release")
        self.specs.pop(req_id, None)

    def stats(self) -> dict:
        st = ServeStats()
        _check(lib().hydro_serve_stats_get(self.ctx.h, C.byref(st)), "hydro_serve_stats_get")
        return {name: getattr(st, name) for name, _ in ServeStats._fields_}

    def stop(self, drain: bool = True) -> None:
        _check(lib().hydro_serve_stop(self.ctx.h, int(drain)), "hydro_serve_stop")
