"""MATLAB -v7.3 MAT-files (HDF5) through mexct_mat_list / _info / _read and
mexct_mat_write_ex (CPU only).

The files come from tests/mat73_writer.py, a writer of the HDF5 structures that
MATLAB's save -v7.3 produces (version 0 superblock behind the 512-byte user
block, version 1 object headers, symbol-table root group) and of the newer
forms (version 2 superblock and object headers, link messages).  Covered:
every numeric class with the MATLAB dimensions reversed, logical, complex
(real part), big-endian types, contiguous / compact / chunked layouts with
ragged edge chunks, one- and two-level chunk B-trees, deflate / shuffle /
Fletcher-32 filters and a per-chunk filter mask, a version 4 single-chunk
layout, header continuation blocks, empty arrays (MATLAB_empty), groups
(structs) and MATLAB's #refs#, and damaged files (an error status, never a
crash).  Written here: -v7.3 files read back, appends (to the library's own
files and to files in MATLAB's layout), and the format rules.
"""
import numpy as np
import pytest

from mat73_writer import DEFLATE, FLETCHER32, SHUFFLE, Mat73Writer

F = np.float32


def _vars(rng):
    return {
        "a_double": rng.standard_normal((5, 3)),
        "b_single": rng.standard_normal((4, 3, 2)).astype(np.float32),
        "c_int16": rng.integers(-3000, 3000, (7, 1)).astype(np.int16),
        "d_uint8": rng.integers(0, 255, (2, 9)).astype(np.uint8),
        "e_int64": rng.integers(-2 ** 40, 2 ** 40, (3, 2)).astype(np.int64),
        "f_uint32": rng.integers(0, 2 ** 31, (1, 6)).astype(np.uint32),
        "g_logical": rng.integers(0, 2, (3, 3)).astype(bool),
    }


@pytest.mark.parametrize("new_style", [False, True], ids=["v0-superblock", "v2-superblock"])
def test_contiguous_variables_of_every_class(lib, tmp_path, new_style):
    from mexct import _lib, fileio

    rng = np.random.default_rng(1)
    vs = _vars(rng)
    w = Mat73Writer(new_style=new_style)
    for name, arr in vs.items():
        w.add(name, arr)
    w.add("s_char", np.frombuffer("scan".encode("utf-16-le"), np.uint16).reshape(1, 4),
          mclass="char")
    w.add_group("t_struct")
    w.add_group("#refs#", mclass=None)
    p = tmp_path / "v73.mat"
    w.save(p)
    assert fileio.mat_list(p) == sorted(list(vs) + ["s_char", "t_struct"])
    for name, arr in vs.items():
        got = fileio.read_mat(p, name)
        assert got.shape == arr.shape and got.dtype == np.float32
        np.testing.assert_array_equal(got, arr.astype(np.float64).astype(np.float32))
    np.testing.assert_array_equal(fileio.read_mat(p), vs["a_double"].astype(np.float32))
    for name in ("s_char", "t_struct"):
        with pytest.raises(_lib.MexctError) as ei:
            fileio.read_mat(p, name)
        assert ei.value.status == _lib.ERR_UNSUPPORTED
    with pytest.raises(_lib.MexctError) as ei:
        fileio.read_mat(p, "nope")
    assert ei.value.status == _lib.ERR_ARG


FILTERS = [(), (DEFLATE,), (SHUFFLE, DEFLATE), (SHUFFLE, DEFLATE, FLETCHER32)]


@pytest.mark.parametrize("filters", FILTERS, ids=["none", "deflate", "shuffle+deflate",
                                                  "shuffle+deflate+fletcher32"])
@pytest.mark.parametrize("levels", [1, 2])
def test_chunked_with_ragged_edges(lib, tmp_path, filters, levels):
    """A 37 x 29 x 5 single volume in 2 x 8 x 16 chunks (file order 5 x 29 x 37):
    partial chunks on every face; a sinogram-like double array besides."""
    from mexct import fileio

    rng = np.random.default_rng(2)
    vol = rng.standard_normal((37, 29, 5)).astype(np.float32)
    sino = rng.uniform(0, 1e5, (24, 10, 7))
    w = Mat73Writer()
    w.add("vol", vol, layout="chunked", chunks=[2, 8, 16], filters=filters, levels=levels)
    w.add("sino", sino, layout="chunked", chunks=[3, 10, 24], filters=filters, levels=levels)
    p = tmp_path / "chunked.mat"
    w.save(p)
    np.testing.assert_array_equal(fileio.read_mat(p, "vol"), vol)
    np.testing.assert_array_equal(fileio.read_mat(p, "sino"), sino.astype(np.float32))


def test_filter_mask_and_single_chunk_layouts(lib, tmp_path):
    """One chunk stored without its deflate step (filter mask bit set), and
    version 4 layouts holding one chunk, deflated or not; compact data."""
    from mexct import fileio

    rng = np.random.default_rng(3)
    a = rng.standard_normal((16, 12)).astype(np.float32)
    w = Mat73Writer(new_style=True)
    w.add("masked", a, layout="chunked", chunks=[4, 8], filters=(SHUFFLE, DEFLATE),
          skip_mask_chunk=(4, 8))
    w.add("single_deflated", a, layout="single", filters=(DEFLATE,))
    w.add("single_plain", a, layout="single")
    w.add("small", np.array([[1.5, -2.0, 3.25]]), layout="compact")
    p = tmp_path / "single.mat"
    w.save(p)
    for name in ("masked", "single_deflated", "single_plain"):
        np.testing.assert_array_equal(fileio.read_mat(p, name), a)
    np.testing.assert_array_equal(fileio.read_mat(p, "small"), np.array([[1.5, -2.0, 3.25]], F))


@pytest.mark.parametrize("new_style", [False, True], ids=["v1-headers", "v2-headers"])
def test_big_endian_complex_and_continuation_blocks(lib, tmp_path, new_style):
    """Big-endian integers and doubles; a complex array reads as its real part;
    the MATLAB_class attribute in a continuation block of the object header."""
    from mexct import fileio

    rng = np.random.default_rng(4)
    i32 = rng.integers(-2 ** 30, 2 ** 30, (6, 5)).astype(np.int32)
    f64 = rng.standard_normal((3, 4, 2))
    z = rng.standard_normal((5, 4)) + 1j * rng.standard_normal((5, 4))
    w = Mat73Writer(new_style=new_style)
    w.add("be_int32", i32, be=True)
    w.add("be_double", f64, be=True, layout="chunked", chunks=[1, 3, 2], filters=(DEFLATE,))
    w.add("cplx", z, continuation=True)
    w.add("cplx_chunked", z.astype(np.complex64), layout="chunked", chunks=[2, 3],
          filters=(SHUFFLE, DEFLATE))
    p = tmp_path / "be.mat"
    w.save(p)
    np.testing.assert_array_equal(fileio.read_mat(p, "be_int32"), i32.astype(F))
    np.testing.assert_array_equal(fileio.read_mat(p, "be_double"), f64.astype(F))
    np.testing.assert_array_equal(fileio.read_mat(p, "cplx"), z.real.astype(F))
    np.testing.assert_array_equal(fileio.read_mat(p, "cplx_chunked"),
                                  z.astype(np.complex64).real)


def test_empty_array_and_scan_sized_names(lib, tmp_path):
    """An empty MATLAB array (MATLAB_empty: the data are its dimensions) has its
    dimensions and no elements; many variables in the symbol table."""
    from mexct import fileio

    w = Mat73Writer()
    w.add("empty", None, mclass="double", empty_dims=[0, 3])
    names = ["view_%03d" % i for i in range(40)]
    for i, n in enumerate(names):
        w.add(n, np.full((2, 2), i, np.float32))
    p = tmp_path / "many.mat"
    w.save(p)
    assert fileio.mat_list(p) == sorted(["empty"] + names)
    e = fileio.read_mat(p, "empty")
    assert e.shape == (0, 3)
    for i, n in enumerate(names):
        np.testing.assert_array_equal(fileio.read_mat(p, n), np.full((2, 2), i, F))


def test_two_level_group_btree(lib, tmp_path):
    """A root group whose symbol table spans a two-level B-tree (as MATLAB's files
    get past a few hundred variables): every variable listed and read."""
    from mexct import fileio

    w = Mat73Writer()
    names = ["p%03d" % i for i in range(30)]
    for i, n in enumerate(names):
        w.add(n, np.full((1, 3), i, np.float32))
    p = tmp_path / "tree2.mat"
    w.save(p, per_node=4)
    assert fileio.mat_list(p) == names
    for i, n in enumerate(names):
        np.testing.assert_array_equal(fileio.read_mat(p, n), np.full((1, 3), i, F))


def test_dense_groups_and_missing_superblock_are_reported(lib, tmp_path):
    from mexct import _lib, fileio

    w = Mat73Writer(new_style=True)
    w.add("x", np.ones((2, 2), np.float32))
    p = tmp_path / "dense.mat"
    w.save(p, dense=True)
    with pytest.raises(_lib.MexctError) as ei:
        fileio.mat_list(p)
    assert ei.value.status == _lib.ERR_UNSUPPORTED
    q = tmp_path / "header_only.mat"
    q.write_bytes(b"MATLAB 7.3 MAT-file, Platform: GLNXA64".ljust(512, b" ") + b"\0" * 64)
    with pytest.raises(_lib.MexctError) as ei:
        fileio.read_mat(q)
    assert ei.value.status == _lib.ERR_IO
    assert "no HDF5 superblock" in _lib.last_error()


def test_unsupported_variable_leaves_the_others_readable(lib, tmp_path):
    """A variable stored with an HDF5 feature the reader does not follow (here a
    version 4 chunk index other than a single chunk) is listed and reports why;
    the file's other variables read as usual."""
    from mexct import _lib, fileio

    a = np.arange(12, dtype=F).reshape(3, 4)
    w = Mat73Writer(new_style=True)
    w.add("good", a)
    w.add("odd", a, layout="single")
    p = tmp_path / "odd.mat"
    w.save(p)
    raw = bytearray(p.read_bytes())
    # the single-chunk layout message: version 4, class 2, flags, 3 dims of 4 bytes,
    # then the index type (1) -> 3 (fixed array)
    i = raw.index(bytes([4, 2, 0, 3, 4]))
    assert raw[i + 5 + 12] == 1
    raw[i + 5 + 12] = 3
    p.write_bytes(bytes(raw))
    assert fileio.mat_list(p) == ["good", "odd"]
    np.testing.assert_array_equal(fileio.read_mat(p, "good"), a)
    with pytest.raises(_lib.MexctError) as ei:
        fileio.read_mat(p, "odd")
    assert ei.value.status == _lib.ERR_UNSUPPORTED
    assert "chunk index" in _lib.last_error()


def test_damaged_files_fail_cleanly(lib, tmp_path):
    """Truncations and seeded byte corruptions of a chunked, deflated file give
    a status (an error, or data when the damage misses every structure read),
    never a crash or a hang."""
    from mexct import _lib, fileio

    rng = np.random.default_rng(5)
    w = Mat73Writer()
    w.add("vol", rng.standard_normal((20, 18, 6)).astype(np.float32), layout="chunked",
          chunks=[3, 8, 8], filters=(SHUFFLE, DEFLATE), levels=2)
    w.add("b", rng.standard_normal((4, 4)))
    good = tmp_path / "good.mat"
    w.save(good)
    raw = good.read_bytes()
    bad = tmp_path / "bad.mat"
    outcomes = {"ok": 0, "error": 0}
    for cut in list(range(0, len(raw), max(1, len(raw) // 60))) + [len(raw) - 1]:
        bad.write_bytes(raw[:cut])
        try:
            fileio.read_mat(bad, "vol")
            outcomes["ok"] += 1
        except _lib.MexctError as e:
            assert e.status in (_lib.ERR_IO, _lib.ERR_UNSUPPORTED, _lib.ERR_ARG)
            outcomes["error"] += 1
    for _ in range(300):
        b = bytearray(raw)
        for _ in range(int(rng.integers(1, 4))):
            b[int(rng.integers(512, len(b)))] = int(rng.integers(0, 256))
        bad.write_bytes(bytes(b))
        try:
            fileio.mat_list(bad)
            fileio.read_mat(bad, "vol")
            outcomes["ok"] += 1
        except _lib.MexctError as e:
            assert e.status in (_lib.ERR_IO, _lib.ERR_UNSUPPORTED, _lib.ERR_ARG)
            outcomes["error"] += 1
    assert outcomes["error"] > 0


def test_v73_writer_roundtrip_and_appends(lib, tmp_path):
    """-v7.3 files written here: MATLAB's header and superblock position; 40
    appended variables (the root group over several symbol table nodes), an
    empty array, all read back; the Level 5 default is unchanged."""
    from mexct import _lib, fileio

    rng = np.random.default_rng(6)
    p = tmp_path / "w73.mat"
    a = rng.standard_normal((17, 9, 5)).astype(F)
    fileio.write_mat(p, "recon", a, format="v7.3")
    raw = p.read_bytes()
    assert raw.startswith(b"MATLAB 7.3 MAT-file") and raw[512:520] == b"\x89HDF\r\n\x1a\n"
    assert fileio.mat_list(p) == ["recon"]
    np.testing.assert_array_equal(fileio.read_mat(p, "recon"), a)
    names = ["v%02d" % i for i in range(40)]
    for i, n in enumerate(names):
        fileio.write_mat(p, n, np.full((3, i + 1), i, F), append=True)  # the file's format
    fileio.write_mat(p, "empty", np.zeros((0, 4), F), append=True)
    assert fileio.mat_list(p) == sorted(["recon", "empty"] + names)
    for i, n in enumerate(names):
        np.testing.assert_array_equal(fileio.read_mat(p, n), np.full((3, i + 1), i, F))
    np.testing.assert_array_equal(fileio.read_mat(p, "recon"), a)
    assert fileio.read_mat(p, "empty").shape == (0, 4)
    with pytest.raises(_lib.MexctError) as ei:
        fileio.write_mat(p, "recon", a, append=True)  # the name is taken
    assert ei.value.status == _lib.ERR_ARG
    with pytest.raises(_lib.MexctError) as ei:
        fileio.write_mat(p, "x", a, append=True, format="v5")  # not into an HDF5 file
    assert ei.value.status == _lib.ERR_ARG
    q = tmp_path / "v5.mat"
    fileio.write_mat(q, "x", a)
    assert q.read_bytes().startswith(b"MATLAB 5.0 MAT-file")


def test_append_to_a_matlab_layout_file(lib, tmp_path):
    """A variable appended to a file in MATLAB's layout (its structs and #refs#
    kept); files with a newer superblock are refused for appending."""
    from mexct import _lib, fileio

    rng = np.random.default_rng(7)
    d = rng.standard_normal((6, 4))
    w = Mat73Writer()
    w.add("data", d)
    w.add("vol", rng.standard_normal((8, 8, 3)).astype(F), layout="chunked", chunks=[2, 4, 4],
          filters=(SHUFFLE, DEFLATE))
    w.add_group("meta")
    w.add_group("#refs#", mclass=None)
    p = tmp_path / "ml.mat"
    w.save(p)
    vol = fileio.read_mat(p, "vol")
    b = rng.standard_normal((5, 5)).astype(F)
    fileio.write_mat(p, "added", b, append=True)
    assert fileio.mat_list(p) == ["added", "data", "meta", "vol"]
    np.testing.assert_array_equal(fileio.read_mat(p, "data"), d.astype(F))
    np.testing.assert_array_equal(fileio.read_mat(p, "vol"), vol)
    np.testing.assert_array_equal(fileio.read_mat(p, "added"), b)
    w2 = Mat73Writer(new_style=True)
    w2.add("x", np.ones((2, 2), F))
    r = tmp_path / "new.mat"
    w2.save(r)
    with pytest.raises(_lib.MexctError) as ei:
        fileio.write_mat(r, "y", b, append=True)
    assert ei.value.status == _lib.ERR_UNSUPPORTED
