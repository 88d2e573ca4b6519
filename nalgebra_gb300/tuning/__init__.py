"""Per-size-bucket tile table of the ragged Cholesky launch.

The library sorts a ragged batch into size buckets and runs one persistent
launch per bucket with the bucket's tile (threads per matrix, panel width).
``autotune`` measures every tile on every bucket on the current GPU
(``nacu_ragged_autotune``) and writes the table to ``ragged_cholesky.json``
beside this file; ``apply`` installs a saved table, and the library loader
applies the saved table on load.
"""
from __future__ import annotations

import ctypes as C
import json
import os

TABLE_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ragged_cholesky.json")


def layout(lib):
    nb, nt = 8, 4
    hi = (C.c_int32 * nb)()
    th = (C.c_int32 * nt)()
    pw = (C.c_int32 * nt)()
    lib.nacu_ragged_tuning_layout(hi, th, pw)
    return list(hi), [{"threads": th[t], "nb": pw[t]} for t in range(nt)]


def autotune(per_bucket: int = 1000, nrhs: int = 4, flags: int = 0, save: bool = True, stream: int = 0,
             path: str | None = None) -> dict:
    """Time every tile on every bucket, install the fastest, optionally save."""
    from .. import _lib

    lib = _lib.load()
    buckets, tiles = layout(lib)
    table = (C.c_int32 * len(buckets))()
    ms = (C.c_double * (len(buckets) * len(tiles)))()
    _lib.check(lib.nacu_ragged_autotune(per_bucket, nrhs, flags, table, ms, C.c_void_p(stream)),
               "nacu_ragged_autotune")
    res = {
        "bucket_hi": buckets,
        "tiles": tiles,
        "table": list(table),
        "ms": [[ms[b * len(tiles) + t] for t in range(len(tiles))] for b in range(len(buckets))],
        "per_bucket": per_bucket,
        "nrhs": nrhs,
    }
    if save:
        with open(path or TABLE_PATH, "w") as f:
            json.dump(res, f, indent=1)
    return res


def apply(lib=None, path: str | None = None) -> list | None:
    """Install the saved table (if any); returns it."""
    p = path or TABLE_PATH
    if not os.path.exists(p):
        return None
    with open(p) as f:
        table = json.load(f)["table"]
    if lib is None:
        from .. import _lib

        lib = _lib.load()
    arr = (C.c_int32 * len(table))(*table)
    if lib.nacu_ragged_set_tuning(arr, len(table)) != 0:
        return None
    return table


def current(lib=None) -> list:
    if lib is None:
        from .. import _lib

        lib = _lib.load()
    arr = (C.c_int32 * 8)()
    lib.nacu_ragged_get_tuning(arr, 8)
    return list(arr)
