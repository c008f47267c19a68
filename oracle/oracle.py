"""ctypes binding of the CPU oracle (oracle/ce_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, bench.py's CPU baseline and
__graft_entry__.smoke() as the checker.  The engine never imports it.

The oracle reads the raw config keys itself (a minimal `key = value` reader,
no validation -- the engine's parser is checked separately), so the two sides
share nothing but the input text and arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libce_oracle.so"
F32, I32 = np.float32, np.int32


def build(force: bool = False) -> Path:
    newest = max((HERE / f).stat().st_mtime for f in ("ce_oracle.c", "ce_oracle_eig.h", "ce_oracle64.h"))
    if force or not LIB.exists() or LIB.stat().st_mtime < newest:
        subprocess.run(["make", "-s", "-C", str(HERE), "-B" if force else "all"], check=True)
    return LIB


class oc_cfg(C.Structure):
    _fields_ = [("ns", C.c_int32), ("nd", C.c_int32), ("nw", C.c_int32), ("n_params", C.c_int32),
                ("input_size", C.c_int32), ("dc_instr", C.c_int32), ("u_instr", C.c_int32),
                ("nl_instr", C.c_int32 * 4), ("serial", C.c_int32), ("time", C.c_int32),
                ("duration", C.c_float), ("ref_step_time", C.c_double), ("ref_amplitude", C.c_float),
                ("fit_start", C.c_float), ("fit_end", C.c_float), ("steady_start", C.c_float),
                ("bandwidth", C.c_float), ("damping", C.c_float), ("overshoot", C.c_float), ("sse", C.c_float),
                ("crossover_coeff", C.c_float), ("target_gm", C.c_float), ("target_pm", C.c_float),
                ("target_b", C.c_float), ("eig_fail_err", C.c_float), ("unstable_err", C.c_float),
                ("freq", C.c_int32), ("freq_min", C.c_float), ("freq_max_key", C.c_float),
                ("observer", C.c_int32)]


class oc_der(C.Structure):
    _fields_ = [("ts", C.c_float), ("freq_max", C.c_float), ("fit_t0", C.c_float), ("fit_t1", C.c_float),
                ("crossover", C.c_float), ("nt", C.c_int32), ("cuda_w", C.c_int32), ("info_scoring", C.c_int32),
                ("info_freqresp", C.c_int32), ("info_allmargin", C.c_int32), ("info_modal", C.c_int32),
                ("info_w", C.c_int32), ("fit_start_id", C.c_int32), ("steady_start_id", C.c_int32),
                ("fit_len", C.c_float)]


_FP = C.POINTER(C.c_float)
_IP = C.POINTER(C.c_int32)
_DP = C.POINTER(C.c_double)


class oc_plant(C.Structure):
    _fields_ = [(n, _FP) for n in ("ss_a", "ss_ai", "ss_b", "ss_c", "ss_d", "d_a", "d_ai", "d_bu", "d_bw", "d_c",
                                   "base_params")] + [(n, _IP) for n in ("dc_info", "u_info", "nl_info")]


class oc_ins(C.Structure):
    _fields_ = [("op", C.c_int32), ("col", C.c_int32), ("akind", C.c_int32), ("bkind", C.c_int32),
                ("aval", C.c_float), ("bval", C.c_float)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        i64 = C.c_int64
        L.oracle_sim.argtypes = [C.POINTER(oc_cfg), C.POINTER(oc_plant), i64, _FP, _FP, C.c_int]
        L.oracle_derived.argtypes = [C.POINTER(oc_cfg), C.POINTER(oc_der)]
        L.oracle_derived.restype = None
        L.oracle_sim_kalman.argtypes = [C.POINTER(oc_cfg), C.POINTER(oc_plant), i64, _FP, C.c_int, C.c_int, _FP,
                                        _IP, C.c_int]
        L.oracle_lina.argtypes = [C.POINTER(oc_cfg), C.POINTER(oc_plant), i64, _FP, _FP, C.c_int]
        L.oracle_eigensolve.argtypes = [i64, C.c_int, _FP, _FP, _DP, C.c_int]
        L.oracle_eigensolve.restype = None
        L.oracle_eig_matrix.argtypes = [_DP, C.c_int, _DP, _DP]
        L.oracle64_evaluate.argtypes = [C.POINTER(oc_cfg), C.POINTER(oc_plant), i64, _FP, _FP, _DP, _DP, _DP, _DP,
                                        _DP, _DP, C.c_int]
        L.oracle_set_eig_fused.argtypes = [C.c_int]
        L.oracle_set_eig_fused.restype = None
        L.oracle_modalsetup.argtypes = [C.POINTER(oc_cfg), i64, _FP, _FP, _FP, _FP, _FP, C.c_int]
        L.oracle_modalsetup.restype = None
        L.oracle_modalsolve.argtypes = [C.POINTER(oc_cfg), i64, _FP, _FP, _FP, _FP, C.c_int]
        L.oracle_modalsolve.restype = None
        L.oracle_allmargin.argtypes = [C.POINTER(oc_cfg), C.POINTER(oc_plant), i64, _FP, _FP, _FP, C.c_int]
        L.oracle_evaluate.argtypes = [C.POINTER(oc_cfg), C.POINTER(oc_plant), i64, _FP, _FP, _FP, _FP, _FP, _FP, _FP,
                                      C.c_int]
        L.oracle_plant_grid.argtypes = [C.POINTER(oc_cfg), C.POINTER(oc_plant), _FP, _FP, _FP, _FP, _IP, _FP]
        L.oracle_decode.argtypes = [_IP, C.c_int, C.c_int, _FP, C.c_int, C.POINTER(oc_ins)]
        L.oracle_info_width.argtypes = [C.POINTER(oc_cfg)]
        _lib = L
    return _lib


def default_threads() -> int:
    return int(os.environ.get("CE_ORACLE_THREADS", os.cpu_count() or 1))


def raw_keys(text: str) -> dict:
    kv = {}
    for line in text.splitlines():
        line = line.split("#", 1)[0].strip()
        if not line:
            continue
        k, v = line.split("=", 1)
        kv[k.strip()] = v.strip()
    return kv


def make_cfg(text: str) -> oc_cfg:
    kv = raw_keys(text)
    g = lambda k, d=None: kv.get(k, d)
    c = oc_cfg()
    c.ns, c.nd, c.nw = int(float(g("statespace_dim"))), int(float(g("discrete_dim"))), int(float(g("nonlin_dim")))
    c.n_params, c.input_size = int(float(g("n_params"))), int(float(g("input_size")))
    c.dc_instr, c.u_instr = int(float(g("dc_instructions"))), int(float(g("u_instructions")))
    nl = [int(float(x)) for x in g("nl_instructions", "").split(",") if x.strip()]
    for i, v in enumerate(nl):
        c.nl_instr[i] = v
    c.serial = 1 if g("mode", "batch") == "serial" else 0
    c.time = int(float(g("time")))
    c.duration = float(g("duration", "1.0"))
    c.ref_step_time = float(g("ref_step_time"))
    for k in ("ref_amplitude", "fit_start", "fit_end", "steady_start", "bandwidth", "damping", "overshoot",
              "crossover_coeff", "target_gm", "target_pm", "target_b"):
        setattr(c, k, float(g(k)))
    c.sse = float(g("steady_state_error"))
    c.eig_fail_err = float(g("eig_fail_err", "1.0e18"))
    c.unstable_err = float(g("unstable_err", "1.0e6"))
    c.freq = int(float(g("freq")))
    c.freq_min = float(g("freq_min"))
    c.freq_max_key = float(g("freq_max", "0"))
    c.observer = 1 if g("observer", "luenberger") == "kalman" else 0
    return c


def _f(a):
    return None if a is None else a.ctypes.data_as(_FP)


class Oracle:
    """One round of the reference method on the CPU for a (config text, plant) pair."""

    def __init__(self, config_text: str, plant, round_index: int = 0, threads: int | None = None,
                 eig_fused: bool = False):
        """eig_fused: the eigensolves (LIN_A and the nominal closed loop) fuse each multiply-add into
        one fma, as the engine's fused eigensolve arithmetic does; False: every product and sum is
        rounded, the reference's arithmetic."""
        self.eig_fused = bool(eig_fused)
        self.cfg = make_cfg(config_text)
        self.threads = threads or default_threads()
        c = self.cfg
        nd, nw, npar = c.nd, c.nw, c.n_params
        arr = {}
        for name, size in (("discrete_a", nd * nd), ("discrete_a_i", nd * nd), ("discrete_bu", nd),
                           ("discrete_bw", nd * nw), ("discrete_c", nd), ("base_params", npar)):
            a = np.ascontiguousarray(getattr(plant, name), F32).reshape(-1)
            arr[name] = np.ascontiguousarray(a[round_index * size:(round_index + 1) * size])
        for name in ("statespace_a", "statespace_a_i", "statespace_b", "statespace_c", "statespace_d"):
            arr[name] = np.ascontiguousarray(getattr(plant, name), F32).reshape(-1)
        for name in ("dc_info", "u_info", "nl_info"):
            arr[name] = np.ascontiguousarray(getattr(plant, name), I32).reshape(-1)
        self._keep = arr
        p = oc_plant()
        names = dict(ss_a="statespace_a", ss_ai="statespace_a_i", ss_b="statespace_b", ss_c="statespace_c",
                     ss_d="statespace_d", d_a="discrete_a", d_ai="discrete_a_i", d_bu="discrete_bu",
                     d_bw="discrete_bw", d_c="discrete_c", base_params="base_params")
        for f, n in names.items():
            setattr(p, f, arr[n].ctypes.data_as(_FP))
        for n in ("dc_info", "u_info", "nl_info"):
            setattr(p, n, arr[n].ctypes.data_as(_IP))
        self.plant = p
        self.nt = c.ns + c.nd
        self.info_w = lib().oracle_info_width(C.byref(c))
        self.cuda_w = 3 * c.ns + 2 if c.observer else 2 * c.ns + 1

    def ref_config(self):
        """The config fields the reference's kernels read (EngineParams and the table sizes), from
        this oracle's parse and derivation -- for oracle/ref_kernels.py without the engine."""
        from types import SimpleNamespace
        c, d = self.cfg, oc_der()
        lib().oracle_derived(C.byref(c), C.byref(d))
        nt = d.nt
        nl = list(c.nl_instr)
        return SimpleNamespace(
            statespace_dim=c.ns, discrete_dim=c.nd, nonlin_dim=c.nw, total_dim=nt, time=c.time,
            cuda_mx_width=d.cuda_w, info_mx_width=d.info_w, info_scoring=d.info_scoring,
            info_freqresp=d.info_freqresp, eigen_mx_width=2 * nt, lina_mx_width=nt * nt, ata_mx_width=4 * nt * nt,
            atb_mx_width=2 * nt, fit_start_id=d.fit_start_id, steady_start_id=d.steady_start_id, ts=d.ts,
            fit_start=c.fit_start, fit_end=c.fit_end, fit_t0=d.fit_t0, fit_t1=d.fit_t1, unstable_err=c.unstable_err,
            n_params=c.n_params, dc_instructions=c.dc_instr, u_instructions=c.u_instr, nl_instructions=nl,
            nl_instructions_total=sum(nl), ref_step_time=c.ref_step_time, ref_amplitude=c.ref_amplitude)

    def _g(self, cuda_mx):
        g = np.ascontiguousarray(cuda_mx, F32).reshape(-1, self.cuda_w)
        return g, g.shape[0]

    def sim(self, cuda_mx):
        g, n = self._g(cuda_mx)
        y = np.empty((n, self.cfg.time), F32)
        rc = lib().oracle_sim(C.byref(self.cfg), C.byref(self.plant), n, _f(g), _f(y), self.threads)
        if rc:
            raise ValueError(f"oracle decode error (digit {rc - 1})")
        return y

    def sim_kalman(self, rows, literal: bool = False):
        """The Kalman observer loop; `literal`: the reference's own row layout [K, N, R, Q]
        and in-place Joseph product.  Returns (y, first step at which P stopped changing)."""
        rows = np.ascontiguousarray(rows, F32)
        n, w = rows.shape
        y = np.empty((n, self.cfg.time), F32)
        steady = np.empty(n, I32)
        rc = lib().oracle_sim_kalman(C.byref(self.cfg), C.byref(self.plant), n, _f(rows), w, int(literal), _f(y),
                                     steady.ctypes.data_as(_IP), self.threads)
        if rc:
            raise ValueError(f"oracle decode error (digit {rc - 1})")
        return y, steady

    def lina(self, cuda_mx):
        g, n = self._g(cuda_mx)
        out = np.empty((n, self.nt * self.nt), F32)
        rc = lib().oracle_lina(C.byref(self.cfg), C.byref(self.plant), n, _f(g), _f(out), self.threads)
        if rc:
            raise ValueError(f"oracle decode error (digit {rc - 1})")
        return out

    def eigensolve(self, lina, fp64=False):
        lina = np.ascontiguousarray(lina, F32)
        n = lina.shape[0]
        e = np.empty((n, 2 * self.nt), F32)
        e64 = np.empty((n, 2 * self.nt), np.float64)
        lib().oracle_set_eig_fused(int(self.eig_fused))
        lib().oracle_eigensolve(n, self.nt, _f(lina), _f(e), e64.ctypes.data_as(_DP), self.threads)
        return e64 if fp64 else e

    def modalsetup(self, y, eig, info):
        y = np.ascontiguousarray(y, F32)
        eig = np.ascontiguousarray(eig, F32)
        info = np.array(info, F32, copy=True, order="C")
        n = info.shape[0]
        ata = np.empty((n, 4 * self.nt * self.nt), F32)
        atb = np.empty((n, 2 * self.nt), F32)
        lib().oracle_modalsetup(C.byref(self.cfg), n, _f(y), _f(eig), _f(ata), _f(atb), _f(info), self.threads)
        return ata, atb, info

    def modalsolve(self, ata, atb, eig, info):
        info = np.array(info, F32, copy=True, order="C")
        n = info.shape[0]
        lib().oracle_modalsolve(C.byref(self.cfg), n, _f(np.ascontiguousarray(ata, F32)),
                                _f(np.ascontiguousarray(atb, F32)), _f(np.ascontiguousarray(eig, F32)), _f(info),
                                self.threads)
        return info

    def allmargin(self, lina, cuda_mx, info):
        g, n = self._g(cuda_mx)
        info = np.array(info, F32, copy=True, order="C")
        lib().oracle_set_eig_fused(int(self.eig_fused))
        rc = lib().oracle_allmargin(C.byref(self.cfg), C.byref(self.plant), n, _f(np.ascontiguousarray(lina, F32)),
                                    _f(g), _f(info), self.threads)
        if rc:
            raise ValueError("allmargin: plant has no finite nonzero gain at crossover")
        return info

    def evaluate(self, cuda_mx, info_in, diagnostics: bool = False):
        g, n = self._g(cuda_mx)
        info = np.array(info_in, F32, copy=True, order="C").reshape(n, self.info_w)
        nt = self.nt
        d = None
        if diagnostics:
            d = dict(yplant=np.empty((n, self.cfg.time), F32), lina=np.empty((n, nt * nt), F32),
                     eigen=np.empty((n, 2 * nt), F32), ata=np.empty((n, 4 * nt * nt), F32),
                     atb=np.empty((n, 2 * nt), F32))
        dd = d or {}
        lib().oracle_set_eig_fused(int(self.eig_fused))
        rc = lib().oracle_evaluate(C.byref(self.cfg), C.byref(self.plant), n, _f(g), _f(info),
                                   _f(dd.get("yplant")), _f(dd.get("lina")), _f(dd.get("eigen")), _f(dd.get("ata")),
                                   _f(dd.get("atb")), self.threads)
        if rc > 0:
            raise ValueError(f"oracle decode error (digit {rc - 1})")
        if rc < 0:
            raise ValueError("allmargin: plant has no finite nonzero gain at crossover")
        return (info, d) if diagnostics else info


    def evaluate64(self, cuda_mx, info_in):
        """One round in the plain FP64 form of the method (the engine's fp64 precision): the INFO
        rows and the double intermediates ywin (n x fit_steps), summ (n x 3: sum of y over the
        steady window, max, min), lina, eigen, ata, atb."""
        g, n = self._g(cuda_mx)
        info = np.array(info_in, F32, copy=True, order="C").reshape(n, self.info_w)
        nt = self.nt
        d = oc_der()
        lib().oracle_derived(C.byref(self.cfg), C.byref(d))
        fit_steps = int(np.ceil(np.float32(d.fit_len))) if d.fit_len > 0 else 0
        out = dict(ywin=np.empty((n, fit_steps)), summ=np.empty((n, 3)), lina=np.empty((n, nt * nt)),
                   eigen=np.empty((n, 2 * nt)), ata=np.empty((n, 4 * nt * nt)), atb=np.empty((n, 2 * nt)))
        dp = lambda a: a.ctypes.data_as(_DP)
        lib().oracle_set_eig_fused(int(self.eig_fused))
        rc = lib().oracle64_evaluate(C.byref(self.cfg), C.byref(self.plant), n, _f(g), _f(info), dp(out["ywin"]),
                                     dp(out["summ"]), dp(out["lina"]), dp(out["eigen"]), dp(out["ata"]),
                                     dp(out["atb"]), self.threads)
        if rc > 0:
            raise ValueError(f"oracle decode error (digit {rc - 1})")
        if rc < 0:
            raise ValueError("allmargin: plant has no finite nonzero gain at crossover")
        return info, out


def eig_matrix(A: np.ndarray, fused: bool = False):
    A = np.ascontiguousarray(A, np.float64)
    n = A.shape[0]
    wr = np.empty(n)
    wi = np.empty(n)
    lib().oracle_set_eig_fused(int(fused))
    ok = lib().oracle_eig_matrix(A.ctypes.data_as(_DP), n, wr.ctypes.data_as(_DP), wi.ctypes.data_as(_DP))
    return bool(ok), wr + 1j * wi


def decode(info: np.ndarray, dim: int, count: int, base_params: np.ndarray):
    info = np.ascontiguousarray(info, I32).reshape(-1)
    bp = np.ascontiguousarray(base_params, F32).reshape(-1)
    out = (oc_ins * max(count, 1))()
    rc = lib().oracle_decode(info.ctypes.data_as(_IP), dim, count, bp.ctypes.data_as(_FP), int(bp.size), out)
    if rc:
        return rc - 1, None
    return 0, [(o.op, o.col, o.akind, o.bkind, o.aval, o.bval) for o in out[:count]]
