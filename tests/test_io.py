"""File outputs of a registration (include/lc2_io.hpp): the PNG encoder
decodes with zlib to the written pixels, the NRRD writer's header and body
read back, the matrix file has the reference's comma-terminated rows."""
import os
import shutil
import struct
import subprocess
import zlib

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def read_png_gray8(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, width = 8, b"", None
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(kind + body) & 0xffffffff
        if kind == b"IHDR":
            width, height, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert (depth, ctype) == (8, 0)
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(height, width + 1)
    assert np.all(rows[:, 0] == 0)
    return rows[:, 1:]


def read_nrrd(path):
    data = open(path, "rb").read()
    head, body = data.split(b"\n\n", 1)
    fields = dict(line.split(": ", 1) for line in head.decode().splitlines()[1:])
    return fields, np.frombuffer(body, np.float32)


@pytest.fixture(scope="module")
def written(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ missing")
    d = tmp_path_factory.mktemp("io")
    exe = str(d / "io_check")
    subprocess.run(["g++", "-std=c++14", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "io_check.cpp"), "-o", exe], check=True)
    subprocess.run([exe, str(d)], check=True)
    return d


def test_png_roundtrip(written):
    px = read_png_gray8(written / "g.png")
    y, x = np.mgrid[0:23, 0:37]
    np.testing.assert_array_equal(px, (x * 7 + y * 11) & 0xff)


def test_nrrd_header_and_body(written):
    f, body = read_nrrd(written / "v.nrrd")
    assert f["type"] == "float" and f["dimension"] == "3" and f["encoding"] == "raw"
    assert f["sizes"] == "4 3 2"
    assert f["space directions"] == "(1.5,0.25,0) (0,2,0) (0,0,3)"
    assert f["space origin"] == "(-10,20.5,3.25)"
    np.testing.assert_array_equal(body, 0.5 * np.arange(24, dtype=np.float32))


def test_matrix_file(written):
    lines = open(written / "m.mat").read().splitlines()
    assert lines[0] == "1,0,0,2.5," and lines[2] == "0,0,2,0.125," and len(lines) == 4
