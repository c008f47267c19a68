"""The engine's config parser against the REFERENCE's own parser.

tests/golden/config_golden.json holds what the reference's load_config /
derive / make_engine_params (src/config.cu, compiled from the reference tree by
`make -C oracle ref`; generator: tests/golden/make_config_golden.py) returned
for every case in tests/golden/config_cases.py: the derived configuration,
floats stored exactly as hex, or the exception text.  Bit-exact.  CPU only."""
import json
import sys
from pathlib import Path

import pytest

import controllerengine_gb300 as ce

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))
from config_cases import cases  # noqa: E402

GOLDEN = json.loads((HERE / "golden" / "config_golden.json").read_text())
CASES = cases()


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_parser_matches_reference(lib, name):
    ref = GOLDEN[name]
    text = CASES[name]
    if "error" in ref:
        with pytest.raises(ce.ControllerEngineError) as e:
            ce.EngineConfig.parse(text)
        assert str(e.value) == ref["error"]
        return
    mine = ce.EngineConfig.parse(text).as_dict()
    for k, v in ref["config"].items():
        got = mine[k]
        if isinstance(v, str):
            assert float(got).hex() == v, (k, float(got).hex(), v)
        else:
            assert got == v, (k, got, v)


def test_every_case_has_a_fixture():
    assert set(CASES) == set(GOLDEN)
