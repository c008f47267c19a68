"""Base-36 instruction decoder (ref: src/main.cu:317-337, README.md:60-89): known-answer
entries from the documented encoding, and the engine's decoder against the oracle's on
random tables.  Bit-exact.  CPU only."""
import numpy as np
import pytest

import controllerengine_gb300 as ce

STATE, CONST, PREV = 1, 0, 2
BP = np.array([0.5, 10.0, -10.0, 1.0, -1.0, 0.0], np.float32)


def dec(rows, dim):
    rows = np.asarray(rows, np.int32).reshape(-1, dim)
    return ce.decode_instructions(rows, dim, rows.shape[0], BP)


def test_kat_mul_state_state(lib):
    d = dec([[3 * 1296, 0, 0]], 3)[0]
    assert (d["op"], d["col"], d["akind"], d["bkind"]) == (3, 0, STATE, STATE)


def test_kat_clamp_consts(lib):
    d = dec([[0, 5 * 1296 + 3 * 36 + 2, 0]], 3)[0]
    assert (d["op"], d["col"], d["akind"], d["bkind"]) == (5, 1, CONST, CONST)
    assert d["aval"] == np.float32(-10.0) and d["bval"] == np.float32(10.0)


def test_kat_prev_digit_35(lib):
    d = dec([[0, 0, 3 * 1296 + 35 * 36 + 1]], 3)[0]
    assert (d["op"], d["col"], d["akind"], d["bkind"], d["bval"]) == (3, 2, PREV, CONST, np.float32(0.5))


def test_last_nonzero_column_wins(lib):
    d = dec([[3 * 1296, 1 * 1296 + 4, 0]], 3)[0]
    assert (d["op"], d["col"], d["akind"], d["bkind"], d["bval"]) == (1, 1, STATE, CONST, np.float32(1.0))


def test_zero_row_is_skip_and_small_entry_is_op0(lib):
    d = dec([[0, 0, 0], [0, 40, 0]], 3)
    assert d[0]["op"] == 0 and d[0]["col"] == 0
    assert d[1]["op"] == 0 and d[1]["col"] == 1 and d[1]["akind"] == CONST  # digits (1, 4): both checked


def test_op_above_6_kept(lib):
    d = dec([[9 * 1296 + 35 * 36 + 35, 0]], 2)[0]
    assert d["op"] == 9 and d["akind"] == PREV and d["bkind"] == PREV


def test_digit_beyond_n_params_is_an_error(lib):
    with pytest.raises(ce.ControllerEngineError,
                       match=r"instruction digit 7 needs BASE_PARAMS\[6\] but n_params is 6"):
        dec([[1 * 1296 + 7 * 36 + 1, 0]], 2)


def test_first_digit_checked_first(lib):
    with pytest.raises(ce.ControllerEngineError, match=r"instruction digit 20 needs"):
        dec([[1 * 1296 + 20 * 36 + 30, 0]], 2)


def test_matches_oracle_on_random_tables(lib, oracle_mod):
    rng = np.random.default_rng(7)
    for dim in (2, 3, 8, 9):
        rows = np.zeros((64, dim), np.int32)
        for r in range(64):
            k = rng.integers(0, 3)
            for _ in range(k):
                op = rng.integers(0, 9)
                d1 = rng.choice([0, 35, *range(1, 7)])
                d2 = rng.choice([0, 35, *range(1, 7)])
                rows[r, rng.integers(0, dim)] = op * 1296 + d1 * 36 + d2
        mine = ce.decode_instructions(rows, dim, 64, BP)
        rc, ref = oracle_mod.decode(rows, dim, 64, BP)
        assert rc == 0
        got = [(int(m["op"]), int(m["col"]), int(m["akind"]), int(m["bkind"]), np.float32(m["aval"]),
                np.float32(m["bval"])) for m in mine]
        assert got == [(a, b, c, d, np.float32(e), np.float32(f)) for a, b, c, d, e, f in ref]


def test_matches_reference_decoder_golden(lib):
    """tests/golden/decode_golden.json: the reference's own decode_instructions
    (src/main.cu:317-337, built by `make -C oracle ref`; generator
    tests/golden/make_decode_golden.py) on 120 seeded tables.  Bit-exact,
    error texts included."""
    import json
    from pathlib import Path
    cases = json.loads((Path(__file__).parent / "golden" / "decode_golden.json").read_text())
    for t in cases:
        rows = np.array(t["rows"], np.int32).reshape(-1, t["dim"]) if t["count"] else np.zeros((0, t["dim"]), np.int32)
        bp = np.array(t["base_params"], np.float32)[:t["n_params"]]
        if "error" in t:
            with pytest.raises(ce.ControllerEngineError) as e:
                ce.decode_instructions(rows, t["dim"], t["count"], bp)
            assert str(e.value) == t["error"]
            continue
        mine = ce.decode_instructions(rows, t["dim"], t["count"], bp)
        assert len(mine) == len(t["decoded"])
        for m, ref in zip(mine, t["decoded"]):
            assert [int(m["op"]), int(m["col"]), int(m["akind"]), int(m["bkind"])] == ref[:4]
            if ref[4] is not None:
                assert float(m["aval"]).hex() == ref[4] and float(m["bval"]).hex() == ref[5]
