"""The C-ABI library loads and exports every entry point include/controller_engine.h declares.  CPU only."""
import re
import subprocess
from pathlib import Path

import controllerengine_gb300 as ce

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    syms = []
    for h in sorted((ROOT / "include").glob("*.h")):
        for m in re.finditer(r"CE_EXPORT\s+[\w\s\*]+?\b(\w+)\s*\(", h.read_text()):
            syms.append(m.group(1))
    return syms


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert "RunControllerEngine" in syms and len(syms) >= 10
    out = subprocess.run(["nm", "-D", "--defined-only", str(ce.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    for s in syms:
        assert hasattr(lib, s)


def test_no_stray_exports(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(ce.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert exported <= set(declared_symbols()), sorted(exported - set(declared_symbols()))


def test_version_and_error_channel(lib):
    assert b"sm_103a" in lib.ce_version()
    import pytest
    with pytest.raises(ce.ControllerEngineError, match="missing `statespace_dim`"):
        ce.EngineConfig.parse("time = 5\n")


def test_ragged_rejects_before_any_device_work(lib):
    """Configuration checks of ce_ragged_create run before it touches the device."""
    import pytest
    from controllerengine_gb300 import synth
    p = synth.mass_spring(4)
    k = synth.with_kalman(p)
    cfgs = [ce.EngineConfig.parse(p.config_text), ce.EngineConfig.parse(k.config_text)]
    with pytest.raises(ce.ControllerEngineError, match="instance 1: a ragged batch runs the Luenberger observer"):
        ce.Ragged([(cfgs[0], p.plant), (cfgs[1], k.plant)])
    with pytest.raises(ce.ControllerEngineError, match="n_inst must be >= 1"):
        ce.Ragged([])


def test_server_result_buffer_validation():
    """A caller's result buffer for a served request must be a C-contiguous float32 array shaped like
    the request's INFO rows; anything else is refused before the request reaches the library."""
    import numpy as np
    import pytest
    i = np.zeros((5, 7), np.float32)
    assert ce.Server._out(None, i).shape == (5, 7)
    buf = np.empty((5, 7), np.float32)
    assert ce.Server._out(buf, i) is buf
    for bad in (np.empty((5, 7), np.float64), np.empty((4, 7), np.float32), np.empty((7, 5), np.float32).T):
        with pytest.raises(ValueError):
            ce.Server._out(bad, i)
