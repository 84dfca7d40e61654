"""The C ABI library: it loads, exports every entry point that include/tsph.h
declares, and its host-only parts work without a GPU."""

import os
import random
import re
import struct
import subprocess

import numpy as np
import pytest

from tinysph_old_gb300 import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tsph.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tsph_[a-z0-9_]+)\s*\(", text)))


def test_header_and_binding_agree(tsph):
    assert declared_symbols() == sorted(tsph.ABI_SYMBOLS)


def test_library_exports_every_declared_symbol(tsph):
    out = subprocess.run(["nm", "-D", "--defined-only", tsph.library_path()],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (tsph_[a-z0-9_]+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    L = tsph.load()
    for s in declared_symbols():
        assert hasattr(L, s)
    assert L.tsph_abi_version() == 1


def test_create_rejects_bad_arguments(tsph):
    import ctypes as C
    L = tsph.load()
    c = tsph._Constants(-1.0, 2.1, 35.0, 1000.0, 0.02, 0.1, 0.01)
    d = tsph._Domain(0.0, 1.0, 0.0, 1.0)
    h = C.c_void_p()
    assert L.tsph_create(C.byref(c), C.byref(d), 0, None, C.byref(h)) == tsph.ERR_ARG
    c = tsph._Constants(0.01, 2.1, 35.0, 1000.0, 0.02, 0.1, 0.01)
    assert L.tsph_create(C.byref(c), C.byref(d), 7, None, C.byref(h)) == tsph.ERR_ARG
    assert b"precision" in L.tsph_last_error()


def test_create_without_gpu_fails_loudly(tsph):
    if tsph.device_count() > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(tsph.TsphError) as e:
        tsph.ParticleSystem(0.01, 2.1, 35.0, 1000.0, 0.02, 0.1, 0.01, (0, 1, 0, 1))
    assert e.value.status == tsph.ERR_CUDA


def _ref_cell(x, x0, of, kh):
    # (int)((x - x_0 + of)/kh) of src/SPH_find_pairs.h:64-65 in IEEE double
    return int((x - x0 + of) / kh)


def _ordered(x):
    b = struct.unpack("<q", struct.pack("<d", x))[0]
    return b if b >= 0 else b ^ 0x7FFFFFFFFFFFFFFF


def _lookup(b, x):
    o = _ordered(x)
    return int(np.searchsorted(b, o, side="right")) - 1


@pytest.mark.parametrize("dp", [0.02, 0.005, 0.0005])
def test_grid_tables_reproduce_reference_cell_index(tsph, dp):
    """The device's cell index (a lookup of the double's bits in the host-built
    tables) equals the reference's FP64 division for every tested double,
    including the doubles adjacent to every cell boundary."""
    c = cases.dam_break_benchmark(dp)
    x0, xm, y0, ym = c.domain
    kh = c.kap * c.h
    of = c.h * 0.273
    ncx, ncy, bx, by = tsph.grid_tables(c.h, c.kap, c.domain)
    assert ncx == int((xm - x0 + of) / kh) + 1
    assert ncy == int((ym - y0 + of) / kh) + 1
    rng = random.Random(7)
    for axis, (b, o0, n) in enumerate(((bx, x0, ncx), (by, y0, ncy))):
        xs = [rng.uniform(o0 - of, o0 - of + n * kh) for _ in range(2000)]
        # both neighbours of every boundary (next double up / down)
        for k in range(0, n + 1, max(1, n // 200)):
            o = int(b[k])
            for dd in (-1, 0, 1):
                oo = o + dd
                bits = oo if oo >= 0 else oo ^ 0x7FFFFFFFFFFFFFFF
                xs.append(struct.unpack("<d", struct.pack("<q", bits))[0])
        for x in xs:
            want = _ref_cell(x, o0, of, kh)
            got = _lookup(b, x)
            if 0 <= want < n:
                assert got == want, (axis, x, want, got)
            else:
                assert got < 0 or got >= n
