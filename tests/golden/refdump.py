"""Reader for the record files written by oracle/ref_build/ref_harness.cpp
(char name[32]; int64 ndim; int64 dims[ndim]; float64 data)."""
from __future__ import annotations

import numpy as np


def read_dump(path: str) -> dict[str, np.ndarray]:
    out = {}
    with open(path, "rb") as f:
        while True:
            name = f.read(32)
            if len(name) < 32:
                break
            nd = int(np.frombuffer(f.read(8), dtype="<i8")[0])
            dims = np.frombuffer(f.read(8 * nd), dtype="<i8")
            n = int(np.prod(dims)) if nd else 1
            data = np.frombuffer(f.read(8 * n), dtype="<f8").reshape(tuple(int(d) for d in dims))
            out[name.rstrip(b"\0").decode()] = data.copy()
    return out
