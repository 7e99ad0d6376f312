"""Scanner data files (CPU): MAT-file Level 5 and VFF readers / writers.

MAT-files written by scipy.io.savemat (compressed and not, several classes),
hand-built compressed elements at zlib levels 0, 1 and 9 (stored, fixed and
dynamic Huffman blocks, long overlapping matches), a hand-built big-endian file,
the library's own writer read back by scipy, and VFF files with a GE-style
header in 8, 16 and 32 bits.
"""
import struct
import zlib

import numpy as np
import pytest

sio = pytest.importorskip("scipy.io")


def _mat_elements(tmp_path, arrays):
    """Level 5 data elements of `arrays` as scipy writes them uncompressed."""
    p = tmp_path / "plain.mat"
    sio.savemat(str(p), arrays, do_compression=False)
    return p.read_bytes()[128:]


def test_scipy_files_compressed_and_plain(lib, tmp_path):
    from mexct import fileio

    rng = np.random.default_rng(0)
    arrays = {
        "vol": rng.standard_normal((7, 5, 3)),                      # double, 3-D
        "sino": rng.standard_normal((6, 4)).astype(np.float32),     # single
        "counts": rng.integers(-3000, 3000, (5, 9)).astype(np.int16),
        "mask": rng.integers(0, 2, (4, 4)).astype(bool),            # logical
        "bytes": rng.integers(0, 255, (3, 8)).astype(np.uint8),
        "sad": np.float64(1000.0),
        "label": "not numeric",
    }
    for comp in (False, True):
        p = tmp_path / ("c%d.mat" % comp)
        sio.savemat(str(p), arrays, do_compression=comp)
        assert set(fileio.mat_list(p)) == set(arrays)
        for name, a in arrays.items():
            if name == "label":
                with pytest.raises(Exception):
                    fileio.read_mat(p, name)
                continue
            got = fileio.read_mat(p, name)
            want = np.atleast_2d(np.asarray(a, dtype=np.float64))
            assert got.shape == want.shape, name
            np.testing.assert_array_equal(got, want.astype(np.float32), err_msg=name)
        # no name: the first numeric variable in the file
        first = [n for n in fileio.mat_list(p) if n != "label"][0]
        np.testing.assert_array_equal(fileio.read_mat(p), fileio.read_mat(p, first))


@pytest.mark.parametrize("level", [0, 1, 9])
@pytest.mark.parametrize("kind", ["random", "runs", "ramp"])
def test_compressed_elements_every_block_kind(lib, tmp_path, level, kind):
    from mexct import fileio

    rng = np.random.default_rng(level)
    if kind == "random":
        a = rng.standard_normal((40, 50)).astype(np.float32)
    elif kind == "runs":  # long runs: matches longer than their distance
        a = np.repeat(rng.integers(0, 4, 60), 97).astype(np.float32).reshape(60, 97)
    else:
        a = np.arange(3000, dtype=np.float32).reshape(50, 60) % 17
    elem = _mat_elements(tmp_path, {"a": a})
    z = zlib.compress(elem, level)
    hdr = (b"MATLAB 5.0 MAT-file".ljust(116, b" ") + b"\0" * 8 + struct.pack("<H", 0x0100)
           + b"IM")
    p = tmp_path / "hand.mat"
    p.write_bytes(hdr + struct.pack("<II", 15, len(z)) + z)
    np.testing.assert_array_equal(fileio.read_mat(p, "a"), a)
    # a damaged stream is an error, not a crash
    bad = bytearray(z)
    bad[len(bad) // 2] ^= 0x5A
    bad[-1] ^= 0xFF
    p.write_bytes(hdr + struct.pack("<II", 15, len(bad)) + bytes(bad))
    from mexct import _lib
    with pytest.raises(_lib.MexctError) as ei:
        fileio.read_mat(p, "a")
    assert ei.value.status == _lib.ERR_IO


def test_big_endian_file(lib, tmp_path):
    """A big-endian Level 5 file: int16 2 x 3 array "be" (small-format name)."""
    from mexct import fileio

    vals = np.array([[1, -2, 300], [-4000, 5, 6]], dtype=np.int16)
    data = vals.astype(">i2").tobytes(order="F")
    body = struct.pack(">II", 6, 8) + struct.pack(">II", 10, 0)       # flags: mxINT16
    body += struct.pack(">II", 5, 8) + struct.pack(">ii", 2, 3)       # dims
    body += struct.pack(">I", (2 << 16) | 1) + b"be\0\0"              # small-format name
    body += struct.pack(">II", 3, len(data)) + data + b"\0" * (-len(data) % 8)
    hdr = (b"MATLAB 5.0 MAT-file".ljust(116, b" ") + b"\0" * 8 + struct.pack(">H", 0x0100)
           + b"MI")
    p = tmp_path / "be.mat"
    p.write_bytes(hdr + struct.pack(">II", 14, len(body)) + body)
    np.testing.assert_array_equal(fileio.read_mat(p, "be"), vals.astype(np.float32))


def test_writer_is_read_by_scipy(lib, tmp_path):
    from mexct import fileio

    rng = np.random.default_rng(3)
    a = rng.standard_normal((6, 5, 4)).astype(np.float32)
    b = rng.standard_normal((3, 7)).astype(np.float32)
    p = tmp_path / "ours.mat"
    fileio.write_mat(p, "recon", a)
    fileio.write_mat(p, "sinogram", b, append=True)
    got = sio.loadmat(str(p))
    np.testing.assert_array_equal(got["recon"], a)
    np.testing.assert_array_equal(got["sinogram"], b)
    assert fileio.mat_list(p) == ["recon", "sinogram"]
    np.testing.assert_array_equal(fileio.read_mat(p, "recon"), a)


def test_unsupported_and_missing(lib, tmp_path):
    from mexct import _lib, fileio

    p = tmp_path / "h5.mat"  # a -v7.3 header with no HDF5 data behind it
    p.write_bytes(b"MATLAB 7.3 MAT-file, Platform: GLNXA64".ljust(512, b" "))
    with pytest.raises(_lib.MexctError) as ei:
        fileio.read_mat(p)
    assert ei.value.status == _lib.ERR_IO
    with pytest.raises(_lib.MexctError) as ei:
        fileio.read_mat(tmp_path / "absent.mat")
    assert ei.value.status == _lib.ERR_IO
    q = tmp_path / "x.mat"
    fileio.write_mat(q, "x", np.ones((2, 2), np.float32))
    with pytest.raises(_lib.MexctError) as ei:
        fileio.read_mat(q, "y")
    assert ei.value.status == _lib.ERR_ARG


def _vff(path, arr, bits, extra=b""):
    X, Y, Z = arr.shape
    hdr = (b"ncaa\ntitle=scan 1;\nrank=3;\ntype=raster;\nformat=slice;\nbits=%d;\nbands=1;\n"
           b"size=%d %d %d;\nspacing=0.1 0.1 0.2;\norigin=0 0 0;\n" % (bits, X, Y, Z)
           + extra + b"\x0c\n")
    dt = {8: ">u1", 16: ">i2", 32: ">f4"}[bits]
    path.write_bytes(hdr + np.asarray(arr).astype(dt).tobytes(order="F"))


@pytest.mark.parametrize("bits", [8, 16, 32])
def test_vff_reader(lib, tmp_path, bits):
    from mexct import fileio

    rng = np.random.default_rng(bits)
    if bits == 8:
        a = rng.integers(0, 256, (9, 7, 4))
    elif bits == 16:
        a = rng.integers(-32768, 32768, (9, 7, 4))
    else:
        a = rng.standard_normal((9, 7, 4)).astype(np.float32)
    # the data begin with a newline byte (0x0a) and the header has unknown keys
    a = np.asarray(a).copy()
    a[0, 0, 0] = {8: 10, 16: 0x0A00, 32: np.frombuffer(b"\x0a\0\0\0", ">f4")[0]}[bits]
    p = tmp_path / ("v%d.vff" % bits)
    _vff(p, a, bits, extra=b"elementsize=0.1;\ny_bin=1;\n")
    vol, sp, b = fileio.read_vff(p)
    assert b == bits and vol.shape == (9, 7, 4)
    np.testing.assert_allclose(sp, [0.1, 0.1, 0.2], rtol=1e-6)
    np.testing.assert_array_equal(vol, np.asarray(a, np.float32))


def test_vff_writer_roundtrip(lib, tmp_path):
    from mexct import _lib, fileio

    rng = np.random.default_rng(9)
    a = rng.standard_normal((12, 10, 6)).astype(np.float32) * 1000
    p = tmp_path / "w.vff"
    fileio.write_vff(p, a, (0.5, 0.5, 1.0), bits=32)
    v, sp, b = fileio.read_vff(p)
    np.testing.assert_array_equal(v, a)
    assert b == 32 and list(sp) == [0.5, 0.5, 1.0]
    fileio.write_vff(p, a * 100, bits=16)  # saturates to int16
    v, _, b = fileio.read_vff(p)
    assert b == 16
    np.testing.assert_array_equal(v, np.clip(np.rint(a * 100), -32768, 32767))
    p.write_bytes(b"P6\n3 3\n255\n" + bytes(27))
    with pytest.raises(_lib.MexctError) as ei:
        fileio.read_vff(p)
    assert ei.value.status == _lib.ERR_IO
