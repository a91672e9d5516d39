"""Locates (and on first use builds) the in-tree native libraries."""
from __future__ import annotations

import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_NAMES = {"engine": "libpbig_gb300.so", "gen": "libpbig_gen.so", "legacy": "libpbig.a"}
_lock = threading.Lock()
_built = False


def lib_path(which: str) -> str:
    """Path of a native library, building the tree once per process if the
    file is missing or was built for another architecture."""
    global _built
    p = os.path.join(_BUILD, _NAMES[which])
    with _lock:
        if not _built:
            from . import build as _b
            stamp_ok = _b._stamp_ok(_BUILD)
            if not (os.path.exists(p) and stamp_ok):
                _b.build(with_oracle=False)
            _built = True
    if not os.path.exists(p):
        raise RuntimeError(f"native library {p} is missing and could not be built")
    return p
