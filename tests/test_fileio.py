"""xerus's binary data-file format (misc::save_to_file / load_from_file,
include/xerus/misc/fileIO.h:103-162) through the C ABI.

The CPU tests encode and decode host cores only (no device call): the bytes the
library writes must equal, byte for byte, the files the reference wrote for
the same tensors (tests/golden/fileio.npz, oracle/ref/golden_driver.cpp
case_fileio). The GPU test round-trips a device tensor through a file.
"""
import os
import shutil

import numpy as np
import pytest

from xerus_gb300 import _lib


@pytest.fixture(scope="module")
def xg():
    if not os.path.exists(_lib.LIB_PATH):
        if not (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
            pytest.skip("nvcc not available to build libxtt.so")
        from xerus_gb300 import build
        build.build()
    import xerus_gb300
    return xerus_gb300


def _cores(g, name, op):
    dims, ranks, flat = g[f"{name}_dims"], g[f"{name}_ranks"], g[f"{name}_cores"]
    out, off = [], 0
    for k, n in enumerate(dims):
        shp = (ranks[k], n, n, ranks[k + 1]) if op else (ranks[k], n, ranks[k + 1])
        sz = int(np.prod(shp))
        out.append(flat[off:off + sz].reshape(shp))
        off += sz
    assert off == flat.size
    return out


def _header_flags(raw):
    """(canonicalized, corePosition) as the reference wrote them (TTNetwork stream, ttNetwork.cpp:1454-1468)."""
    body = raw[raw.index(b"Format: Binary\n") + len(b"Format: Binary\n"):]
    assert int.from_bytes(body[:8], "little") == 1
    return bool(body[8]), int.from_bytes(body[9:17], "little")


@pytest.mark.parametrize("name,op", [("x", False), ("y", False), ("z", False), ("A", True)])
def test_encode_matches_reference_bytes(xg, golden, name, op):
    g = golden("fileio")
    raw = bytes(g[f"{name}_bytes"])
    canon, pos = _header_flags(raw)
    got = xg.file_encode(_cores(g, name, op), is_operator=op, canonicalized=canon, core_position=pos)
    assert got == raw


@pytest.mark.parametrize("name,op", [("x", False), ("y", False), ("z", False), ("A", True)])
def test_decode_reference_file(xg, golden, name, op):
    g = golden("fileio")
    raw = bytes(g[f"{name}_bytes"])
    cores, is_op, canon, pos = xg.file_decode(raw)
    assert is_op == op
    assert (canon, pos) == _header_flags(raw)
    want = _cores(g, name, op)
    assert len(cores) == len(want)
    for a, b in zip(cores, want):
        assert a.shape == b.shape
        assert np.array_equal(a, b)  # bit-exact: the file holds the doubles verbatim


def test_reference_flags_of_the_golden_files(golden):
    """The reference's canonical flags: random and move_core results canonical, core at 0 and 2."""
    g = golden("fileio")
    assert _header_flags(bytes(g["x_bytes"])) == (True, 0)
    assert _header_flags(bytes(g["y_bytes"])) == (True, 2)
    assert _header_flags(bytes(g["z_bytes"])) == tuple(bool(v) if i == 0 else int(v) for i, v in enumerate(g["z_canon"]))


def test_sparse_representation_decodes(xg, golden):
    """A component stored sparse (Tensor representation 2, tensor.cpp:1781-1802) reads as the same dense values."""
    g = golden("fileio")
    raw = bytearray(bytes(g["x_bytes"]))
    cores = _cores(g, "x", False)
    # locate the second component's dense block: header + version 1 + order + dims + representation 1
    c = cores[1]
    block = b"".join(int(v).to_bytes(8, "little") for v in (1, 3, *c.shape, 1)) + c.astype("<f8").tobytes()
    at = bytes(raw).index(block)
    nz = [(i, v) for i, v in enumerate(c.ravel()) if i % 3 != 1]  # drop a third: those read back as 0
    sparse = b"".join(int(v).to_bytes(8, "little") for v in (1, 3, *c.shape, 2, len(nz)))
    sparse += b"".join(int(i).to_bytes(8, "little") + np.float64(v).astype("<f8").tobytes() for i, v in nz)
    raw[at:at + len(block)] = sparse
    got, _, _, _ = xg.file_decode(bytes(raw))
    want = c.ravel().copy()
    want[1::3] = 0.0
    assert np.array_equal(got[1].ravel(), want)
    for k in (0, 2, 3):
        assert np.array_equal(got[k], cores[k])


@pytest.mark.parametrize("cut", [10, 60, 200, -9, -1])
def test_truncated_file_is_an_argument_error(xg, golden, cut):
    raw = bytes(golden("fileio")["x_bytes"])
    with pytest.raises(xg.XttError) as e:
        xg.file_decode(raw[:cut])
    assert e.value.code == 1  # XTT_ERR_ARGUMENT


def test_other_file_kinds_are_rejected(xg, golden):
    raw = bytes(golden("fileio")["x_bytes"])
    with pytest.raises(xg.XttError):
        xg.file_decode(raw.replace(b"TTNetwork<false>", b"Tensor", 1))
    with pytest.raises(xg.XttError):
        xg.file_decode(raw.replace(b"Format: Binary", b"Format: TSV", 1))
    with pytest.raises(xg.XttError):
        xg.file_decode(raw + b"\0")


def test_random_round_trip(xg):
    rng = np.random.default_rng(7)
    for op in (False, True):
        dims, ranks = [2, 5, 3, 4, 2], [1, 2, 4, 5, 3, 1]
        cores = [rng.standard_normal((ranks[k], n, n, ranks[k + 1]) if op else (ranks[k], n, ranks[k + 1]))
                 for k, n in enumerate(dims)]
        raw = xg.file_encode(cores, is_operator=op, canonicalized=True, core_position=3)
        back, is_op, canon, pos = xg.file_decode(raw)
        assert (is_op, canon, pos) == (op, True, 3)
        for a, b in zip(back, cores):
            assert np.array_equal(a, b)


@pytest.mark.gpu
def test_device_save_load(xg, golden, tmp_path):
    """save_to_file of a device tensor writes the reference's bytes; load_from_file restores cores and flags."""
    g = golden("fileio")
    for name, op in (("y", False), ("A", True)):
        raw = bytes(g[f"{name}_bytes"])
        src = tmp_path / f"{name}_ref.xrs"
        src.write_bytes(raw)
        t = xg.load_from_file(str(src))
        assert isinstance(t, xg.TTOperator if op else xg.TTTensor)
        assert (t.canonicalized, t.corePosition) == _header_flags(raw)
        for a, b in zip(t.get_cores(), _cores(g, name, op)):
            assert np.array_equal(a, b)
        out = tmp_path / f"{name}_out.xrs"
        xg.save_to_file(t, str(out))
        assert out.read_bytes() == raw
