"""CPU checks of the C++ host mirror (include/titgpu.hpp) and the .ttdb
writer (include/titgpu_data.hpp): the host-only logic runs in a small C++
program, and its storage is read back here with SQLite and a zstd decoder.
The titwcsph-style driver is built and fails cleanly without a GPU."""

from __future__ import annotations

import ctypes
import ctypes.util
import os
import pathlib
import sqlite3
import struct
import subprocess

import numpy as np
import pytest

from titsolver_gb300 import build as gpu_build

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _zstd_lib():
    name = ctypes.util.find_library("zstd")
    for cand in ([name] if name else []) + ["libzstd.so.1"]:
        try:
            lib = ctypes.CDLL(cand)
        except OSError:
            continue
        lib.ZSTD_getFrameContentSize.restype = ctypes.c_ulonglong
        lib.ZSTD_getFrameContentSize.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
        lib.ZSTD_decompress.restype = ctypes.c_size_t
        lib.ZSTD_decompress.argtypes = [ctypes.c_void_p, ctypes.c_size_t,
                                        ctypes.c_void_p, ctypes.c_size_t]
        lib.ZSTD_isError.restype = ctypes.c_uint
        lib.ZSTD_isError.argtypes = [ctypes.c_size_t]
        return lib
    return None


def decode_raw_frame(blob: bytes) -> bytes:
    """Parse a zstd frame of raw blocks (RFC 8878 3.1.1): the writer's own
    layout, checked field by field."""
    assert struct.unpack_from("<I", blob, 0)[0] == 0xFD2FB528
    assert blob[4] == 0xE0  # 8-byte content size, single segment
    size = struct.unpack_from("<Q", blob, 5)[0]
    pos, out = 13, bytearray()
    while True:
        hdr = int.from_bytes(blob[pos:pos + 3], "little")
        pos += 3
        last, btype, bsize = hdr & 1, (hdr >> 1) & 3, hdr >> 3
        assert btype == 0 and bsize <= 128 * 1024
        out += blob[pos:pos + bsize]
        pos += bsize
        if last:
            break
    assert pos == len(blob) and len(out) == size
    return bytes(out)


def decode(blob: bytes) -> bytes:
    raw = decode_raw_frame(blob)
    lib = _zstd_lib()
    if lib is not None:  # the real decoder agrees
        n = lib.ZSTD_getFrameContentSize(blob, len(blob))
        assert n == len(raw)
        dst = ctypes.create_string_buffer(max(int(n), 1))
        got = lib.ZSTD_decompress(dst, len(dst), blob, len(blob))
        assert not lib.ZSTD_isError(got) and got == n
        assert dst.raw[:got] == raw
    return raw


def type_id(kind: int, rank: int, dim: int) -> int:
    return (kind + 1) | rank << 8 | dim << 16


@pytest.fixture(scope="module")
def mirror_check(tmp_path_factory, gpu_lib):
    exe = tmp_path_factory.mktemp("mirror") / "mirror_check"
    lib_dir = gpu_build.OUT_DIR
    cmd = ["g++", "-std=c++20", "-O1", "-Wall", "-Wextra", "-Werror",
           "-I", str(ROOT / "include"), str(ROOT / "tests" / "cpp" / "mirror_check.cpp"),
           "-L", str(lib_dir), "-ltitgpu", f"-Wl,-rpath,{lib_dir}", "-ldl", "-pthread",
           "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_mirror_host_logic_and_storage(mirror_check, tmp_path):
    db = tmp_path / "particles.ttdb"
    res = subprocess.run([str(mirror_check), str(db)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    assert res.stdout.strip() == "ok"
    con = sqlite3.connect(db)
    tables = {r[0] for r in con.execute("SELECT name FROM sqlite_master WHERE type='table'")}
    assert {"Settings", "DataSeries", "DataFrames", "DataArrays"} <= tables
    assert con.execute("SELECT max_series FROM Settings").fetchall() == [(1,)]
    series = con.execute("SELECT id, name FROM DataSeries").fetchall()
    assert [s[1] for s in series] == ["second"]
    frames = con.execute("SELECT id, time FROM DataFrames WHERE series_id = ? ORDER BY id",
                         (series[0][0],)).fetchall()
    assert [f[1] for f in frames] == [0.0, 0.5]
    rows = {name: (t, n, decode(data)) for name, t, n, data in con.execute(
        "SELECT name, type, size, data FROM DataArrays WHERE frame_id = ?", (frames[0][0],))}
    assert rows["r"][:2] == (type_id(9, 1, 2), 3)
    np.testing.assert_array_equal(np.frombuffer(rows["r"][2], "<f8"),
                                  [1.0, 2.0, 3.0, 4.0, 5.0, 6.0])
    assert rows["rho"][:2] == (type_id(9, 0, 1), 3)
    assert rows["f32"][:2] == (type_id(8, 0, 1), 2)
    np.testing.assert_array_equal(np.frombuffer(rows["f32"][2], "<f4"), [1.5, -2.0])
    assert rows["ids"][:2] == (type_id(4, 0, 1), 4)
    np.testing.assert_array_equal(np.frombuffer(rows["ids"][2], "<i4"), [7, 8, 9, 10])
    big = np.frombuffer(rows["big"][2], "<f8")
    np.testing.assert_array_equal(big, 0.5 * np.arange(40000))
    assert rows["empty"][1] == 0 and rows["empty"][2] == b""
    # The frame written in the background.
    (rho2,) = con.execute("SELECT data FROM DataArrays WHERE frame_id = ?",
                          (frames[1][0],)).fetchone()
    np.testing.assert_array_equal(np.frombuffer(decode(rho2), "<f8"), [1000.0, 1001.5, 999.25])
    # Deleting the series cascades to its frames and arrays.
    con.execute("PRAGMA foreign_keys = ON")
    con.execute("DELETE FROM DataSeries")
    assert con.execute("SELECT COUNT(*) FROM DataArrays").fetchone() == (0,)
    con.close()


def test_driver_builds_and_fails_cleanly_without_device(gpu_lib):
    exe = gpu_build.build_host()["titwcsph_gpu"]
    assert exe.exists() and os.access(exe, os.X_OK)
    res = subprocess.run([str(exe), "--nx", "8", "--steps", "1"], capture_output=True,
                         text=True, timeout=120)
    if res.returncode == 0:
        pytest.skip("a CUDA device is visible")
    assert res.returncode == 1
    assert "no CUDA device" in res.stderr
    bad = subprocess.run([str(exe), "--bogus"], capture_output=True, text=True, timeout=60)
    assert bad.returncode == 1 and "unknown option" in bad.stderr
    # The face-wall setup builds its surface and containment on the host
    # and fails only at the device.
    fw = subprocess.run([str(exe), "--faces", "--fp32c", "--nx", "8"], capture_output=True,
                        text=True, timeout=60)
    assert fw.returncode == 1 and "no CUDA device" in fw.stderr
