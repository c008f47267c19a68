"""Generates tests/golden/decode_golden.json by running the REFERENCE's own
decode_instructions (src/main.cu:317-337, built into oracle/_ref/libref_main.so
by `make -C oracle ref`) on seeded random instruction tables, including rows
with several nonzero entries, op codes above 6, SKIP rows, digits 0 / 35 /
constants, negative entries, and digits beyond n_params (errors)."""
import ctypes as C
import json
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


class Ins(C.Structure):
    _fields_ = [("op", C.c_int), ("col", C.c_int), ("akind", C.c_int), ("bkind", C.c_int), ("aval", C.c_float),
                ("bval", C.c_float)]


def tables(seed=11):
    rng = np.random.default_rng(seed)
    out = []
    for case in range(120):
        dim = int(rng.choice([1, 2, 3, 5, 8, 9]))
        count = int(rng.integers(0, 9))
        n_params = int(rng.integers(1, 35))
        bp = rng.standard_normal(34).astype(np.float32)
        rows = np.zeros((max(count, 1), dim), np.int32)
        for r in range(count):
            for _ in range(int(rng.integers(0, 3))):
                op = int(rng.choice([0, 1, 2, 3, 4, 5, 6, 7, 30]))
                lim = n_params + 1 if rng.random() < 0.9 else 35
                d1 = int(rng.choice([0, 35, int(rng.integers(1, lim))]))
                d2 = int(rng.choice([0, 35, int(rng.integers(1, lim))]))
                v = op * 1296 + d1 * 36 + d2
                if rng.random() < 0.03:
                    v = -int(rng.integers(1, 3000))
                rows[r, int(rng.integers(0, dim))] = v
        out.append(dict(dim=dim, count=count, n_params=n_params, base_params=bp.tolist(),
                        rows=rows[:count].reshape(-1).tolist()))
    return out


def main():
    lib = C.CDLL(str(HERE.parents[1] / "oracle" / "_ref" / "libref_main.so"))
    res = []
    for t in tables():
        rows = np.array(t["rows"] or [0], np.int32)
        bp = np.array(t["base_params"], np.float32)
        out = (Ins * max(t["count"], 1))()
        err = C.create_string_buffer(512)
        rc = lib.ref_decode(rows.ctypes.data_as(C.POINTER(C.c_int)), t["dim"], t["count"],
                            bp.ctypes.data_as(C.POINTER(C.c_float)), t["n_params"], out, err, 512)
        rec = dict(t)
        if rc:
            rec["error"] = err.value.decode()
        else:
            ops = []
            for k, o in enumerate(out[:t["count"]]):
                op = [o.op, o.col, o.akind, o.bkind, float(np.float32(o.aval)).hex(), float(np.float32(o.bval)).hex()]
                # a negative entry makes the reference read below BASE_PARAMS for a SKIP / no-op
                # instruction: the value is never used, so it is not part of the fixture
                if min(t["rows"][k * t["dim"]:(k + 1) * t["dim"]], default=0) < 0 and o.op <= 0:
                    op[4] = op[5] = None
                ops.append(op)
            rec["decoded"] = ops
        res.append(rec)
    (HERE / "decode_golden.json").write_text(json.dumps(res) + "\n")
    print(len(res), "tables,", sum("error" in r for r in res), "errors")


if __name__ == "__main__":
    main()
