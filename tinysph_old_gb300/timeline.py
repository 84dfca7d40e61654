"""Per-kernel time of a replayed CUDA-graph step, from CUPTI kernel activity
records (``libtsph_trace.so``, built from ``csrc/tsph_trace.cpp`` where CUPTI
is installed).

A graph step's kernels cannot be bracketed by CUDA events one by one, and
with programmatic dependent launch a kernel may start (and wait) before its
predecessor ends.  Two figures per kernel are therefore reported:

* ``us``: its own start-to-end time per step (overlapping ones included);
* ``exclusive_us``: the part of the step's busy time attributed to it: from
  the later of its start and the end of everything before it, to its end.
  These add up to the step's busy time (the union of the kernels' intervals).
"""

from __future__ import annotations

import ctypes as C
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(PKG, "libtsph_trace.so")


def kernel_name(mangled: str) -> str:
    """The kernel's identifier (``k_...``) from its mangled name."""
    m = re.search(r"(\d+)(k_)", mangled)
    if not m:
        return mangled[:64]
    n = int(m.group(1))
    return mangled[m.start(2):m.start(2) + n]


class Timeline:
    """start() / stop() around synchronised work; records() afterwards."""

    def __init__(self):
        if not os.path.exists(LIB):
            raise FileNotFoundError(f"{LIB} is not built (CUPTI not installed?)")
        self._L = C.CDLL(LIB)
        L = self._L
        for f in ("tsph_trace_start", "tsph_trace_stop", "tsph_trace_count"):
            getattr(L, f).restype = C.c_int
            getattr(L, f).argtypes = []
        L.tsph_trace_get.restype = C.c_int
        L.tsph_trace_get.argtypes = [C.c_int, C.c_char_p, C.c_int,
                                     C.POINTER(C.c_ulonglong), C.POINTER(C.c_ulonglong),
                                     C.POINTER(C.c_uint)]

    def start(self):
        rc = self._L.tsph_trace_start()
        if rc:
            raise RuntimeError(f"tsph_trace_start failed ({rc})")

    def stop(self):
        rc = self._L.tsph_trace_stop()
        if rc:
            raise RuntimeError(f"tsph_trace_stop failed ({rc})")

    def records(self):
        """[(name, start_ns, end_ns, stream)] in start order."""
        out = []
        buf = C.create_string_buffer(1024)
        s, e, st = C.c_ulonglong(), C.c_ulonglong(), C.c_uint()
        for i in range(self._L.tsph_trace_count()):
            if self._L.tsph_trace_get(i, buf, len(buf), C.byref(s), C.byref(e), C.byref(st)):
                continue
            out.append((kernel_name(buf.value.decode(errors="replace")), s.value, e.value,
                        st.value))
        out.sort(key=lambda r: r[1])
        return out


def split(records, steps: int, prefix: str = "k_"):
    """Per-kernel time per step of the records whose name starts with
    `prefix` (the library's kernels): {"busy_us", "by_kernel": {name:
    {"us", "exclusive_us", "launches"}}}."""
    by = {}
    busy = 0.0
    last_end = None
    for name, s, e, _ in records:
        # kernels of a conditional node whose body did not run come with no
        # timestamps
        if not name.startswith(prefix) or s == 0:
            continue
        d = by.setdefault(name, {"us": 0.0, "exclusive_us": 0.0, "launches": 0})
        d["us"] += (e - s) * 1e-3
        d["launches"] += 1
        lo = s if last_end is None else max(s, last_end)
        excl = max(0, e - lo) * 1e-3
        d["exclusive_us"] += excl
        busy += excl
        last_end = e if last_end is None else max(last_end, e)
    for d in by.values():
        d["us"] /= steps
        d["exclusive_us"] /= steps
        d["launches"] /= steps
    order = sorted(by.items(), key=lambda kv: -kv[1]["exclusive_us"])
    return {"busy_us": busy / steps, "by_kernel": dict(order)}
