"""Python mirror of the reference's interface, on top of the C ABI.

The reference is driven through files (ControllerEngine.config + *.bin) and one
call, RunControllerEngine() (ref: src/main.cu:592-602).  This module offers:

* ``run_controller_engine(workdir)`` -- that call, unchanged, in a directory;
* ``EngineConfig.parse(text)`` -- the reference's config parser (same keys,
  defaults and error messages, ref: src/config.cu:106-244) with the derived sizes;
* ``decode_instructions(...)`` -- the base-36 instruction decoder
  (ref: src/main.cu:317-337);
* ``PlantFiles`` -- the .bin file set as numpy arrays (read/write);
* ``Session`` -- a device-resident plant with ``evaluate`` (host arrays),
  ``evaluate_diagnostics`` and ``evaluate_device`` (device pointers), the
  in-memory form of one RunControllerEngine round.

Errors raise ``ControllerEngineError`` carrying the library's message.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _ffi

F32 = np.float32
I32 = np.int32


class ControllerEngineError(RuntimeError):
    pass


def _lib():
    return _ffi.load_library()


def _check(rc: int):
    if rc != 0:
        raise ControllerEngineError(_ffi.last_error(_lib()))


def _fptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == F32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ffi._FP)


def _iptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == I32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ffi._IP)


class EngineConfig:
    """A parsed ControllerEngine.config with its derived sizes."""

    def __init__(self, raw: _ffi.ce_config):
        self.raw = raw

    @classmethod
    def parse(cls, text: str, filename: str = "ControllerEngine.config") -> "EngineConfig":
        raw = _ffi.ce_config()
        _check(_lib().ce_parse_config(text.encode(), filename.encode(), C.byref(raw)))
        return cls(raw)

    def __getattr__(self, name):
        raw = self.__dict__["raw"]
        v = getattr(raw, name)
        if name == "nl_instructions":
            return list(v)
        return v

    def as_dict(self) -> dict:
        out = {}
        for name, _ in _ffi.ce_config._fields_:
            v = getattr(self.raw, name)
            out[name] = list(v) if name == "nl_instructions" else v
        return out


def decode_instructions(info: np.ndarray, dim: int, count: int, base_params: np.ndarray) -> np.ndarray:
    """Decode `count` rows of width `dim`; returns a structured array (op, col, akind, bkind, aval, bval)."""
    info = np.ascontiguousarray(info, dtype=I32).reshape(-1)
    bp = np.ascontiguousarray(base_params, dtype=F32).reshape(-1)
    out = (_ffi.ce_instruction * max(count, 1))()
    _check(_lib().ce_decode_instructions(_iptr(info) if info.size else None, dim, count,
                                         _fptr(bp) if bp.size else None, int(bp.size), out))
    dt = np.dtype([("op", I32), ("col", I32), ("akind", I32), ("bkind", I32), ("aval", F32), ("bval", F32)])
    arr = np.frombuffer(bytes(out), dtype=dt)[:count].copy()
    return arr


PLANT_FILES = (
    ("statespace_a", "STATESPACE_A.bin", F32), ("statespace_a_i", "STATESPACE_A_I.bin", F32),
    ("statespace_b", "STATESPACE_B.bin", F32), ("statespace_c", "STATESPACE_C.bin", F32),
    ("statespace_d", "STATESPACE_D.bin", F32),
    ("discrete_a", "DISCRETE_A.bin", F32), ("discrete_a_i", "DISCRETE_A_I.bin", F32),
    ("discrete_bu", "DISCRETE_BU.bin", F32), ("discrete_bw", "DISCRETE_BW.bin", F32),
    ("discrete_c", "DISCRETE_C.bin", F32), ("base_params", "BASE_PARAMS.bin", F32),
    ("dc_info", "DC_INFO.bin", I32), ("u_info", "U_INFO.bin", I32), ("nl_info", "NL_INFO.bin", I32),
)


@dataclass
class PlantFiles:
    """The reference's plant/observer/instruction .bin set (compact row-major, flattened)."""

    statespace_a: np.ndarray
    statespace_a_i: np.ndarray
    statespace_b: np.ndarray
    statespace_c: np.ndarray
    statespace_d: np.ndarray
    discrete_a: np.ndarray
    discrete_a_i: np.ndarray
    discrete_bu: np.ndarray
    discrete_bw: np.ndarray
    discrete_c: np.ndarray
    base_params: np.ndarray
    dc_info: np.ndarray
    u_info: np.ndarray
    nl_info: np.ndarray

    def __post_init__(self):
        for name, _, dt in PLANT_FILES:
            setattr(self, name, np.ascontiguousarray(getattr(self, name), dtype=dt).reshape(-1))

    def write(self, directory: str | os.PathLike):
        d = Path(directory)
        for name, fname, _ in PLANT_FILES:
            getattr(self, name).tofile(d / fname)

    @classmethod
    def read(cls, directory: str | os.PathLike) -> "PlantFiles":
        d = Path(directory)
        return cls(**{name: np.fromfile(d / fname, dtype=dt) for name, fname, dt in PLANT_FILES})

    def round_slice(self, cfg: EngineConfig, r: int) -> "PlantFiles":
        """The plant of round r of a serial (stacked) file set."""
        nd, nw, npar = cfg.discrete_dim, cfg.nonlin_dim, cfg.n_params
        kw = {name: getattr(self, name) for name, _, _ in PLANT_FILES}
        for name, size in (("discrete_a", nd * nd), ("discrete_a_i", nd * nd), ("discrete_bu", nd),
                           ("discrete_bw", nd * nw), ("discrete_c", nd), ("base_params", npar)):
            kw[name] = getattr(self, name)[r * size:(r + 1) * size]
        return PlantFiles(**kw)

    def ce_plant(self) -> _ffi.ce_plant:
        p = _ffi.ce_plant()
        for name, _, dt in PLANT_FILES:
            a = getattr(self, name)
            setattr(p, name, _iptr(a) if dt == I32 else _fptr(a))
        return p


class Ragged:
    """Instances of different configurations and plants evaluated together
    (ce_ragged_create): one launch per stage over the candidates of all instances.
    `instances` is a list of (EngineConfig, PlantFiles); `evaluate` takes one
    (cuda_mx, info_mx) pair per instance (any row counts, zero included) and returns
    the INFO rows per instance, each bit-identical to its own session's."""

    def __init__(self, instances: list):
        self.configs = [c for c, _ in instances]
        self._plants = [p for _, p in instances]  # keeps the arrays alive for the call
        k = len(instances)
        cfgs = (_ffi.ce_config * k)(*[c.raw for c in self.configs])
        pls = (_ffi.ce_plant * k)(*[p.ce_plant() for p in self._plants])
        self._h = C.c_void_p()
        _check(_lib().ce_ragged_create(k, cfgs, pls, C.byref(self._h)))

    def evaluate(self, rows: list) -> list:
        if len(rows) != len(self.configs):
            raise ValueError(f"{len(rows)} row sets for {len(self.configs)} instances")
        gs, infos, counts = [], [], []
        for c, (g, i) in zip(self.configs, rows):
            g = np.ascontiguousarray(g, dtype=F32).reshape(-1, c.cuda_mx_width)
            n = g.shape[0]
            i = np.zeros((n, c.info_mx_width), F32) if i is None else i
            gs.append(g.reshape(-1))
            infos.append(np.ascontiguousarray(i, dtype=F32).reshape(n, c.info_mx_width).reshape(-1))
            counts.append(n)
        g_all = np.concatenate(gs) if gs else np.zeros(0, F32)
        i_all = np.concatenate(infos) if infos else np.zeros(0, F32)
        out = np.empty_like(i_all)
        nc = (C.c_int64 * len(counts))(*counts)
        _check(_lib().ce_ragged_evaluate(self._h, nc, _fptr(g_all) if g_all.size else None,
                                         _fptr(i_all) if i_all.size else None, _fptr(out) if out.size else None))
        res, off = [], 0
        for c, n in zip(self.configs, counts):
            w = c.info_mx_width
            res.append(out[off:off + n * w].reshape(n, w))
            off += n * w
        return res

    def prepare(self, n_cand):
        """Fix the candidate counts per instance for evaluate_device (ce_ragged_prepare)."""
        nc = (C.c_int64 * len(n_cand))(*[int(k) for k in n_cand])
        _check(_lib().ce_ragged_prepare(self._h, nc))

    def evaluate_device(self, d_cuda_mx: int, d_info_in: int, d_info_out: int, stream: int = 0):
        """Enqueue one evaluation of the prepared counts on device rows packed instance after
        instance (ce_ragged_evaluate_device); no synchronisation, no allocation."""
        _check(_lib().ce_ragged_evaluate_device(self._h, C.c_void_p(d_cuda_mx), C.c_void_p(d_info_in),
                                                C.c_void_p(d_info_out), C.c_void_p(stream)))

    @property
    def tuning(self) -> dict:
        t = _ffi.ce_ragged_tuning()
        _check(_lib().ce_ragged_get_tuning(self._h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in t._fields_}

    def set_tuning(self, sim_lanes: int = 0, instance_order: int = 0, eig_blocks_per_sm: int = 0,
                   sim_width: int = 0):
        """Launch settings (none changes a result): sim_lanes 4 (the wide form) or 1; instance_order
        0 (grouped by dimension class, program and horizon), 1 (the caller's order) or 2 (dealt by
        horizon); eig_blocks_per_sm; sim_width 0 (each warp at its candidates' dimension class) or 8
        (every candidate at the padded 8/8 width).  0 takes the default."""
        t = _ffi.ce_ragged_tuning(sim_lanes, instance_order, eig_blocks_per_sm, sim_width, 0.0)
        _check(_lib().ce_ragged_set_tuning(self._h, C.byref(t)))

    def autotune(self, d_cuda_mx: int, d_info_in: int, d_info_out: int, stream: int = 0) -> dict:
        t = _ffi.ce_ragged_tuning()
        _check(_lib().ce_ragged_autotune(self._h, C.c_void_p(d_cuda_mx), C.c_void_p(d_info_in),
                                         C.c_void_p(d_info_out), C.c_void_p(stream), C.byref(t)))
        return {k: getattr(t, k) for k, _ in t._fields_}

    def evaluate_packed(self, n_cand, cuda_mx: np.ndarray, info_in: np.ndarray) -> np.ndarray:
        """The C ABI's form: n_cand[i] candidates of instance i, the rows packed instance
        after instance at each instance's widths (flat float32 arrays); returns the INFO rows
        packed the same way."""
        counts = [int(k) for k in n_cand]
        g = np.ascontiguousarray(cuda_mx, dtype=F32).reshape(-1)
        i = np.ascontiguousarray(info_in, dtype=F32).reshape(-1)
        if g.size != sum(k * c.cuda_mx_width for k, c in zip(counts, self.configs)) or \
                i.size != sum(k * c.info_mx_width for k, c in zip(counts, self.configs)):
            raise ValueError("packed rows do not match the candidate counts")
        out = np.empty_like(i)
        nc = (C.c_int64 * len(counts))(*counts)
        _check(_lib().ce_ragged_evaluate(self._h, nc, _fptr(g) if g.size else None, _fptr(i) if i.size else None,
                                         _fptr(out) if out.size else None))
        return out

    @property
    def kernel_launches(self) -> int:
        return int(_lib().ce_ragged_kernel_launches(self._h))

    def set_profiling(self, on: bool):
        _check(_lib().ce_ragged_set_profiling(self._h, 1 if on else 0))

    def stage_times(self) -> dict:
        """{stage: (milliseconds summed, launches)} since profiling was switched on."""
        ms = (C.c_double * _ffi.NUM_STAGES)()
        n = (C.c_int64 * _ffi.NUM_STAGES)()
        _check(_lib().ce_ragged_stage_times(self._h, ms, n))
        return {name: (ms[i], n[i]) for i, name in enumerate(_ffi.STAGE_NAMES)}

    def close(self):
        if self._h:
            _lib().ce_ragged_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Session:
    """Plant + config resident on the current CUDA device (ce_session_create)."""

    def __init__(self, config: EngineConfig, plant: PlantFiles, n_plants: int = 1, precision: str = "mixed"):
        self.config = config
        self._plant = plant  # keeps the arrays alive for the call
        self._h = C.c_void_p()
        raw = config.raw
        _check(_lib().ce_session_create(C.byref(raw), C.byref(plant.ce_plant()), n_plants, C.byref(self._h)))
        self.set_precision(precision)

    def set_precision(self, precision: str):
        code = {"mixed": _ffi.PRECISION_MIXED, "fp64": _ffi.PRECISION_FP64,
                "compensated": _ffi.PRECISION_COMPENSATED,
                "compensated_traj64": _ffi.PRECISION_COMPENSATED_TRAJ64,
                "compensated_df": _ffi.PRECISION_COMPENSATED_DF}[precision]
        _check(_lib().ce_session_set_precision(self._h, code))
        self.precision = precision

    @property
    def eig_arith(self) -> str:
        """Arithmetic of the FP64 eigensolves: "fused" (one DFMA per multiply-add, the default) or
        "separate" (every product and sum rounded, the reference's host arithmetic)."""
        v = C.c_int32()
        _check(_lib().ce_session_get_eig_arith(self._h, C.byref(v)))
        return {_ffi.EIG_ARITH_SEPARATE: "separate", _ffi.EIG_ARITH_FUSED: "fused"}[v.value]

    def set_eig_arith(self, arith: str):
        code = {"separate": _ffi.EIG_ARITH_SEPARATE, "fused": _ffi.EIG_ARITH_FUSED}[arith]
        _check(_lib().ce_session_set_eig_arith(self._h, code))

    def close(self):
        if self._h:
            _lib().ce_session_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def kernel_launches(self) -> int:
        return int(_lib().ce_session_kernel_launches(self._h))

    @property
    def sim_kernel(self) -> str:
        """"specialised" (compiled for the plant's instruction program) or "table"."""
        k = int(_lib().ce_session_sim_kernel(self._h))
        return {_ffi.SIM_TABLE: "table", _ffi.SIM_SPECIALISED: "specialised"}[k]

    def set_sim_kernel(self, kind: str):
        k = {"table": _ffi.SIM_TABLE, "specialised": _ffi.SIM_SPECIALISED}[kind]
        _check(_lib().ce_session_set_sim_kernel(self._h, k))

    @property
    def sim_log(self) -> str:
        return _lib().ce_session_sim_log(self._h).decode()

    def specialised_source(self, plant: int = 0) -> str:
        size = C.c_int64(0)
        _check(_lib().ce_sim_specialised_source(self._h, plant, None, 0, C.byref(size)))
        buf = C.create_string_buffer(size.value)
        _check(_lib().ce_sim_specialised_source(self._h, plant, buf, size.value, C.byref(size)))
        return buf.value.decode()

    @property
    def tuning(self) -> dict:
        t = _ffi.ce_tuning()
        _check(_lib().ce_session_get_tuning(self._h, C.byref(t)))
        return {f: getattr(t, f) for f, _ in t._fields_}

    def set_tuning(self, eig_lanes: int = 0, eig_blocks_per_sm: int = 0, chunks: int = 0):
        t = _ffi.ce_tuning(eig_lanes, eig_blocks_per_sm, chunks, 0.0)
        _check(_lib().ce_session_set_tuning(self._h, C.byref(t)))

    def autotune(self, n: int, d_cuda_mx: int, d_info_in: int, d_info_out: int, stream: int = 0,
                 plant_index: int = 0) -> dict:
        """Time launch settings on this batch (device pointers) and keep the fastest (ce_session_autotune)."""
        t = _ffi.ce_tuning()
        _check(_lib().ce_session_autotune(self._h, plant_index, n, C.c_void_p(d_cuda_mx), C.c_void_p(d_info_in),
                                          C.c_void_p(d_info_out), C.c_void_p(stream), C.byref(t)))
        return {f: getattr(t, f) for f, _ in t._fields_}

    def set_profiling(self, on: bool):
        _check(_lib().ce_session_set_profiling(self._h, 1 if on else 0))

    def stage_times(self) -> dict:
        """{stage: (milliseconds summed, launches)} since profiling was switched on."""
        ms = (C.c_double * _ffi.NUM_STAGES)()
        n = (C.c_int64 * _ffi.NUM_STAGES)()
        _check(_lib().ce_session_stage_times(self._h, ms, n))
        return {name: (ms[i], n[i]) for i, name in enumerate(_ffi.STAGE_NAMES)}

    def _rows(self, cuda_mx, info_in):
        c = self.config
        g = np.ascontiguousarray(cuda_mx, dtype=F32).reshape(-1, c.cuda_mx_width)
        n = g.shape[0]
        if info_in is None:
            info_in = np.zeros((n, c.info_mx_width), F32)
        i = np.ascontiguousarray(info_in, dtype=F32).reshape(n, c.info_mx_width)
        return g, i, n

    def evaluate(self, cuda_mx: np.ndarray, info_in: np.ndarray | None = None, plant_index: int = 0) -> np.ndarray:
        """One round: gains rows [K, L, N] -> INFO rows (input columns passed through)."""
        g, i, n = self._rows(cuda_mx, info_in)
        out = np.empty_like(i)
        _check(_lib().ce_evaluate(self._h, plant_index, n, _fptr(g), _fptr(i), _fptr(out)))
        return out

    def evaluate_diagnostics(self, cuda_mx, info_in=None, plant_index: int = 0, want=("yplant", "lina", "eigen",
                                                                                      "ata", "atb")):
        g, i, n = self._rows(cuda_mx, info_in)
        c = self.config
        nt = c.total_dim
        shapes = {"yplant": (n, c.time), "lina": (n, nt * nt), "eigen": (n, 2 * nt), "ata": (n, 4 * nt * nt),
                  "atb": (n, 2 * nt)}
        arrs = {k: np.empty(shapes[k], F32) for k in want}
        d = _ffi.ce_diagnostics(*[_fptr(arrs.get(k)) for k in ("yplant", "lina", "eigen", "ata", "atb")])
        out = np.empty_like(i)
        _check(_lib().ce_evaluate_diagnostics(self._h, plant_index, n, _fptr(g), _fptr(i), _fptr(out), C.byref(d)))
        return out, arrs

    def evaluate_diagnostics64(self, cuda_mx, info_in=None, plant_index: int = 0,
                               want=("ywin", "summ", "lina", "eigen", "ata", "atb")):
        """Intermediates in double as the session's precision computed them (ce_evaluate_diagnostics64)."""
        g, i, n = self._rows(cuda_mx, info_in)
        c = self.config
        nt = c.total_dim
        shapes = {"ywin": (n, c.fit_steps), "summ": (n, 4), "lina": (n, nt * nt), "eigen": (n, 2 * nt),
                  "ata": (n, 4 * nt * nt), "atb": (n, 2 * nt)}
        arrs = {k: np.empty(shapes[k], np.float64) for k in want}
        dp = lambda a: None if a is None else a.ctypes.data_as(_ffi._DP)
        d = _ffi.ce_diagnostics64(*[dp(arrs.get(k)) for k in ("ywin", "summ", "lina", "eigen", "ata", "atb")])
        out = np.empty_like(i)
        _check(_lib().ce_evaluate_diagnostics64(self._h, plant_index, n, _fptr(g), _fptr(i), _fptr(out), C.byref(d)))
        return out, arrs

    def evaluate_plants(self, cuda_mx: np.ndarray, info_in: np.ndarray | None = None, first_plant: int = 0) -> np.ndarray:
        """One plant per candidate: row c uses plant first_plant + c (ce_evaluate_plants)."""
        g, i, n = self._rows(cuda_mx, info_in)
        out = np.empty_like(i)
        _check(_lib().ce_evaluate_plants(self._h, first_plant, n, _fptr(g), _fptr(i), _fptr(out)))
        return out

    def evaluate_plants_device(self, n: int, d_cuda_mx: int, d_info_in: int, d_info_out: int, stream: int = 0,
                               first_plant: int = 0):
        _check(_lib().ce_evaluate_plants_device(self._h, first_plant, n, C.c_void_p(d_cuda_mx), C.c_void_p(d_info_in),
                                                C.c_void_p(d_info_out), C.c_void_p(stream)))

    def evaluate_device(self, n: int, d_cuda_mx: int, d_info_in: int, d_info_out: int, stream: int = 0,
                        plant_index: int = 0):
        """Enqueue on `stream`: device pointers (ints), no synchronisation."""
        _check(_lib().ce_evaluate_device(self._h, plant_index, n, C.c_void_p(d_cuda_mx), C.c_void_p(d_info_in),
                                         C.c_void_p(d_info_out), C.c_void_p(stream)))


class Request:
    """One submitted request: its buffers stay referenced until `wait` returns."""

    def __init__(self, server: "Server", rid: int, cuda_mx: np.ndarray, info_in: np.ndarray, out: np.ndarray):
        self._server, self.id = server, rid
        self._keep = (cuda_mx, info_in)
        self.out = out

    def wait(self, timeout_ms: int = -1) -> np.ndarray | None:
        """INFO rows of the request, or None if `timeout_ms` passed first."""
        rc = _lib().ce_server_wait(self._server._h, self.id, timeout_ms)
        if rc == _ffi.PENDING:
            return None
        _check(rc)
        self._keep = None
        return self.out


class Server:
    """Continuous-batching front end (ce_server_*): requests of any size, packed per plant into batches of up
    to `max_batch` candidates, `lanes` batches in flight on the GPU."""

    def __init__(self, config: EngineConfig, plant: PlantFiles, n_plants: int = 1, max_batch: int = 0,
                 lanes: int = 0, hbm_budget_bytes: int = 0, max_wait_us: int = 0,
                 models: list | None = None, precision: str = "mixed", max_batch_work: int = 0):
        """One model (config, plant, n_plants), or with `models` a list of such triples
        (ce_server_create_models); requests then name their model in `submit`."""
        models = models or [(config, plant, n_plants)]
        self.configs = [m[0] for m in models]
        self.config = self.configs[0]
        self._plants = [m[1] for m in models]  # keeps the arrays alive for the call
        self._h = C.c_void_p()
        prec = {"mixed": _ffi.PRECISION_MIXED, "fp64": _ffi.PRECISION_FP64,
                "compensated": _ffi.PRECISION_COMPENSATED,
                "compensated_traj64": _ffi.PRECISION_COMPENSATED_TRAJ64,
                "compensated_df": _ffi.PRECISION_COMPENSATED_DF}[precision]
        opt = _ffi.ce_server_options(max_batch, lanes, hbm_budget_bytes, max_wait_us, prec, max_batch_work)
        k = len(models)
        cfgs = (_ffi.ce_config * k)(*[m[0].raw for m in models])
        pls = (_ffi.ce_plant * k)(*[m[1].ce_plant() for m in models])
        nps = (C.c_int32 * k)(*[m[2] for m in models])
        _check(_lib().ce_server_create_models(cfgs, pls, nps, k, C.byref(opt), C.byref(self._h)))

    @staticmethod
    def _out(out, i):
        """The result buffer: the caller's (C-contiguous float32, the INFO rows' shape), or a new one.
        A caller serving many requests passes buffers it reuses, so the result copy does not fault
        in fresh pages."""
        if out is None:
            return np.empty_like(i)
        if out.dtype != F32 or out.shape != i.shape or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float32 array shaped like the INFO rows")
        return out

    def submit(self, cuda_mx: np.ndarray, info_in: np.ndarray | None = None, plant_index: int = 0,
               model: int = 0, out: np.ndarray | None = None) -> Request:
        c = self.configs[model]
        g = np.ascontiguousarray(cuda_mx, dtype=F32).reshape(-1, c.cuda_mx_width)
        n = g.shape[0]
        if info_in is None:
            info_in = np.zeros((n, c.info_mx_width), F32)
        i = np.ascontiguousarray(info_in, dtype=F32).reshape(n, c.info_mx_width)
        out = self._out(out, i)
        rid = C.c_int64()
        _check(_lib().ce_server_submit_model(self._h, model, plant_index, n, _fptr(g), _fptr(i), _fptr(out),
                                             C.byref(rid)))
        return Request(self, rid.value, g, i, out)

    def submit_plants(self, cuda_mx: np.ndarray, info_in: np.ndarray | None = None, first_plant: int = 0,
                      model: int = 0, out: np.ndarray | None = None) -> Request:
        """A Monte Carlo request: row k on plant first_plant + k (ce_server_submit_plants)."""
        c = self.configs[model]
        g = np.ascontiguousarray(cuda_mx, dtype=F32).reshape(-1, c.cuda_mx_width)
        n = g.shape[0]
        if info_in is None:
            info_in = np.zeros((n, c.info_mx_width), F32)
        i = np.ascontiguousarray(info_in, dtype=F32).reshape(n, c.info_mx_width)
        out = self._out(out, i)
        rid = C.c_int64()
        _check(_lib().ce_server_submit_plants(self._h, model, first_plant, n, _fptr(g), _fptr(i), _fptr(out),
                                              C.byref(rid)))
        return Request(self, rid.value, g, i, out)

    def stats(self) -> dict:
        st = _ffi.ce_server_stats()
        _check(_lib().ce_server_get_stats(self._h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in st._fields_}

    def reset_stats(self):
        _check(_lib().ce_server_reset_stats(self._h))

    def close(self):
        if self._h:
            _lib().ce_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def measure_fma_rate(fp64: bool = False) -> float:
    """FMA-issue throughput of the current device, operations per second."""
    v = C.c_double()
    _check(_lib().ce_measure_fma_rate(1 if fp64 else 0, C.byref(v)))
    return v.value


def run_controller_engine(workdir: str | os.PathLike) -> int:
    """Call RunControllerEngine() with `workdir` as the current directory."""
    old = os.getcwd()
    os.chdir(workdir)
    try:
        return int(_lib().RunControllerEngine())
    finally:
        os.chdir(old)
