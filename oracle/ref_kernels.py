"""Runs the reference's own kernels (oracle/_ref/ref_kernels.cubin, built from
src/main.cu by `make -C oracle ref`) on a workload, through the driver-API
runner oracle/ref_shim/ref_kernel_runner.cpp.

TEST INFRASTRUCTURE ONLY.  The constant tables are set as the reference's
init64KB/upload_plant set them (ref: src/main.cu:304-399): compact .bin arrays
scattered into the MAX-padded layout, instruction tables decoded by the
oracle's decoder (itself pinned to the reference's decode_instructions) with
the NL output column remapped to MAX_DISCRETE_DIM.
"""
from __future__ import annotations

import ctypes as C
import struct
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
CUBIN = HERE / "_ref" / "ref_kernels.cubin"
# the same build with the approximate __fdividef read as the correctly rounded quotient (oracle/Makefile)
CUBIN_RN = HERE / "_ref" / "ref_kernels_rn.cubin"
RUNNER = HERE / "_build" / "libref_runner.so"
F32, I32 = np.float32, np.int32


def available() -> bool:
    return CUBIN.exists()


def _runner():
    if not RUNNER.exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "_build/libref_runner.so"], check=True)
    L = C.CDLL(str(RUNNER))
    L.ref_runner_error.restype = C.c_char_p
    return L


def _pad(a, rows, cols, stride, total):
    out = np.zeros(total, F32)
    a = np.asarray(a, F32).reshape(rows, cols) if rows * cols else np.zeros((rows, cols), F32)
    for i in range(rows):
        out[i * stride:i * stride + cols] = a[i]
    return out


def _ops(decoded, count):
    buf = bytearray(24 * count)
    for r, (op, col, ak, bk, av, bv) in enumerate(decoded):
        struct.pack_into("<iiiiff", buf, 24 * r, op, col, ak, bk, av, bv)
    return bytes(buf)


def _tables(cfg, plant, n: int, cuda_w: int):
    """ENGINE bytes, padded constant tables, decoded DC/U/NL records and ref[t]."""
    from oracle import oracle as O
    ns, nd, nw, nt = cfg.statespace_dim, cfg.discrete_dim, cfg.nonlin_dim, cfg.total_dim
    engine = struct.pack("<15i6f", n, cfg.time, ns, nd, nt, cuda_w, cfg.info_mx_width, cfg.info_scoring,
                         cfg.info_freqresp, cfg.eigen_mx_width, cfg.lina_mx_width, cfg.ata_mx_width,
                         cfg.atb_mx_width, cfg.fit_start_id, cfg.steady_start_id, cfg.ts, cfg.fit_start,
                         cfg.fit_end, cfg.fit_t0, cfg.fit_t1, cfg.unstable_err)
    bp = np.asarray(plant.base_params, F32)[:cfg.n_params]
    tabs = [_pad(plant.statespace_a, ns, ns, 8, 64), _pad(plant.statespace_a_i, ns, ns, 8, 64),
            _pad(plant.statespace_b, ns, 1, 1, 8), _pad(plant.statespace_c, 1, ns, 8, 8),
            _pad(plant.statespace_d, 1, 1, 1, 1),
            _pad(plant.discrete_a[:nd * nd], nd, nd, 8, 64), _pad(plant.discrete_a_i[:nd * nd], nd, nd, 8, 64),
            _pad(plant.discrete_bu[:nd], nd, 1, 1, 8), _pad(plant.discrete_bw[:nd * nw], nd, nw, 4, 32),
            _pad(plant.discrete_c[:nd], 1, nd, 8, 8), _pad(bp, 1, cfg.n_params, 34, 34)]
    skip = (0, 0, 0, 0, 0.0, 0.0)
    rc, dc = O.decode(plant.dc_info, nd, cfg.dc_instructions, bp)
    assert rc == 0
    rc, u = O.decode(plant.u_info, ns, cfg.u_instructions, bp)
    assert rc == 0
    nl = [skip] * 32
    row = 0
    info_rows = np.asarray(plant.nl_info, I32).reshape(-1, nd + 1) if cfg.nl_instructions_total else None
    for i in range(nw):
        cnt = cfg.nl_instructions[i]
        rc, ch = O.decode(info_rows[row:row + cnt], nd + 1, cnt, bp)
        assert rc == 0
        for r, ins in enumerate(ch):
            ins = list(ins)
            if ins[1] == nd:
                ins[1] = 8
            nl[i * 8 + r] = tuple(ins)
        row += cnt
    dc = (list(dc) + [skip] * 4)[:4]
    u = (list(u) + [skip] * 4)[:4]
    ref = np.array([0.0 if t < cfg.ref_step_time * cfg.time else cfg.ref_amplitude for t in range(cfg.time)], F32)
    return engine, tabs, _ops(dc, 4), _ops(u, 4), _ops(nl, 32), ref


_fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))


def run(cfg, plant, cuda_mx: np.ndarray, eigen: np.ndarray, info_in: np.ndarray, want_y: bool = True,
        times: dict | None = None):
    """cfg: an engine EngineConfig (its parser is pinned to the reference's).  Returns
    (yplant, lina, ata, atb, info) from the reference kernels (yplant None unless want_y).
    `times`, if given, receives the milliseconds of the three kernels and of the copies."""
    nt = cfg.total_dim
    n = cuda_mx.shape[0]
    engine, tabs, dc, u, nl, ref = _tables(cfg, plant, n, cfg.cuda_mx_width)
    L = _runner()
    tab_ptrs = (C.POINTER(C.c_float) * 11)(*[_fp(t) for t in tabs])
    g = np.ascontiguousarray(cuda_mx, F32)
    e = np.ascontiguousarray(eigen, F32)
    inf = np.ascontiguousarray(info_in, F32)
    y = np.empty((n, cfg.time), F32) if want_y else None
    lina = np.empty((n, nt * nt), F32)
    ata = np.empty((n, 4 * nt * nt), F32)
    atb = np.empty((n, 2 * nt), F32)
    out = np.empty_like(inf)
    tm = np.zeros(5, F32)
    rc = L.ref_run(str(CUBIN).encode(), engine, len(engine), tab_ptrs, dc, u, nl, n,
                   cfg.time, cfg.cuda_mx_width, nt, cfg.info_mx_width, _fp(g), _fp(ref), _fp(e), _fp(inf),
                   _fp(y) if want_y else None, _fp(lina), _fp(ata), _fp(atb), _fp(out), _fp(tm))
    if rc:
        raise RuntimeError(L.ref_runner_error().decode())
    if times is not None:
        times.update(zip(("discrete_solve", "eigensetup", "modalsetup", "h2d", "d2h"), map(float, tm)))
    return y, lina, ata, atb, out


def run_kalman(cfg, plant, rows: np.ndarray, rounded_reciprocal: bool = False):
    """The reference's discrete_solve<Kalman> on rows of its own layout [K(ns), N, R, Q(ns)]
    (2ns+2 floats, given to the kernel as ENGINE.cuda_mx_width).  Returns yplant.  With
    rounded_reciprocal, from the build whose __fdividef is the correctly rounded quotient."""
    rows = np.ascontiguousarray(rows, F32)
    n, w = rows.shape
    assert w == 2 * cfg.statespace_dim + 2
    engine, tabs, dc, u, nl, ref = _tables(cfg, plant, n, w)
    L = _runner()
    tab_ptrs = (C.POINTER(C.c_float) * 11)(*[_fp(t) for t in tabs])
    y = np.empty((n, cfg.time), F32)
    cubin = CUBIN_RN if rounded_reciprocal else CUBIN
    rc = L.ref_run_kalman(str(cubin).encode(), engine, len(engine), tab_ptrs, dc, u, nl, n, cfg.time, w, _fp(rows),
                          _fp(ref), _fp(y))
    if rc:
        raise RuntimeError(L.ref_runner_error().decode())
    return y
