"""HDF5 file I/O of the reference's file path (include/io.h:35-197 and the element-type
dispatch of include/hpdbscan.h:300-356) through the C ABI (hpd_h5_read / hpd_h5_write),
on CPU.

libhdf5 is not available here, so input files are laid out byte by byte by
tests/h5_files.py the way libhdf5 writes them (both its default and its latest file
format), and the library's output is read back and structurally checked by that
module's independent reader.
"""
import os

import numpy as np
import pytest

import h5_files as H

DTYPES = [np.float32, np.float64, np.int8, np.int16, np.int32, np.int64, np.uint8, np.uint16, np.uint32, np.uint64]


@pytest.fixture(scope="module")
def io(engine_lib):
    from hpdbscan_gb300 import hdf5
    return hdf5


def _points(dt, n=57, d=3, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.random((n, d)) * 100 - (50 if np.dtype(dt).kind in "if" else 0)
    return x.astype(dt)


@pytest.mark.parametrize("fmt", ["earliest", "latest"])
@pytest.mark.parametrize("dt", DTYPES, ids=lambda t: np.dtype(t).name)
def test_read_every_element_type(io, tmp_path, fmt, dt):
    a = _points(dt)
    p = str(tmp_path / "x.h5")
    H.write_matrix(p, a, fmt=fmt)
    b = io.read_hdf5(p, "DATA")
    assert b.dtype == a.dtype and np.array_equal(a, b)


@pytest.mark.parametrize("fmt", ["earliest", "latest"])
@pytest.mark.parametrize("kw", [
    dict(big=True),
    dict(layout="compact"),
    dict(layout="chunked", chunk=(8, 2)),
    dict(layout="chunked", chunk=(5, 3), chunks_per_node=3),
    dict(layout="chunked", chunk=(64, 4)),
    dict(split=2),
    dict(big=True, layout="chunked", chunk=(7, 1)),
], ids=["big-endian", "compact", "chunked", "chunked-2-level", "one-chunk", "continuation", "big-chunked"])
def test_read_layouts(io, tmp_path, fmt, kw):
    for dt in (np.float32, np.int16, np.uint64):
        a = _points(dt, n=41)
        p = str(tmp_path / "x.h5")
        H.write_matrix(p, a, fmt=fmt, **kw)
        assert np.array_equal(io.read_hdf5(p, "DATA"), a)


@pytest.mark.parametrize("fmt", ["earliest", "latest"])
def test_read_nested_paths(io, tmp_path, fmt):
    a = _points(np.float64)
    p = str(tmp_path / "x.h5")
    H.write_matrix(p, a, name="group/inner/DATA", fmt=fmt)
    for name in ("group/inner/DATA", "/group/inner/DATA", "group//inner/./DATA"):
        assert np.array_equal(io.read_hdf5(p, name), a)
    with pytest.raises(ValueError, match="^Could not open dataset group/DATA$"):
        io.read_hdf5(p, "group/DATA")
    with pytest.raises(ValueError, match="^Could not open dataset group/inner$"):
        io.read_hdf5(p, "group/inner")  # a group, not a dataset


def test_read_many_entries_and_two_level_group_tree(io, tmp_path):
    f = H.H5("earliest")
    arrays = {f"set{i:03d}": _points(np.float32, n=5 + i, seed=i) for i in range(40)}
    kids = {nm: f.dataset(a) for nm, a in arrays.items()}
    p = str(tmp_path / "many.h5")
    f.finish(kids, p, levels=2)
    for nm, a in arrays.items():
        assert np.array_equal(io.read_hdf5(p, nm), a)
    with pytest.raises(ValueError, match="^Could not open dataset set040$"):
        io.read_hdf5(p, "set040")
    with pytest.raises(ValueError, match="^Could not open dataset aaa$"):
        io.read_hdf5(p, "aaa")


@pytest.mark.parametrize("fmt", ["earliest", "latest"])
def test_unwritten_storage_reads_the_fill_value(io, tmp_path, fmt):
    a = np.zeros((6, 2), np.int32)
    p = str(tmp_path / "x.h5")
    H.write_matrix(p, a, fmt=fmt, unwritten=True, fill=np.int32(-7).tobytes())
    assert np.array_equal(io.read_hdf5(p, "DATA"), np.full((6, 2), -7, np.int32))
    H.write_matrix(p, a, fmt=fmt, unwritten=True)
    assert np.array_equal(io.read_hdf5(p, "DATA"), a)
    H.write_matrix(p, a, fmt=fmt, unwritten=True, layout="chunked", chunk=(4, 2), fill=np.int32(3).tobytes())
    assert np.array_equal(io.read_hdf5(p, "DATA"), np.full((6, 2), 3, np.int32))


def test_empty_matrix(io, tmp_path):
    p = str(tmp_path / "x.h5")
    H.write_matrix(p, np.zeros((0, 3), np.float32))
    b = io.read_hdf5(p, "DATA")
    assert b.shape == (0, 3) and b.dtype == np.float32


def test_user_block(io, tmp_path):
    """A superblock after a 512-byte user block: addresses are relative to the base
    address, the end-of-file address counts from the start of the file."""
    p = str(tmp_path / "x.h5")
    a = _points(np.float32)
    H.write_matrix(p, a)
    # relocate: user block of 512 bytes, base address 512 in the superblock
    raw = bytearray(open(p, "rb").read())
    raw[24:32] = (512).to_bytes(8, "little")
    raw[40:48] = (len(raw) + 512).to_bytes(8, "little")
    with open(p, "wb") as fh:
        fh.write(b"\0" * 512 + raw)
    assert np.array_equal(io.read_hdf5(p, "DATA"), a)
    io.write_hdf5(p, "CLUSTERS", np.arange(57))
    assert np.array_equal(io.read_hdf5(p, "DATA"), a)
    assert np.array_equal(H.read_labels(p, "CLUSTERS"), np.arange(57))


MAT73 = None
try:  # a file written by libhdf5 itself: MATLAB 7.3 format (HDF5 behind a 512-byte user block)
    import scipy.io.matlab as _m
    _p = os.path.join(os.path.dirname(_m.__file__), "tests", "data", "testhdf5_7.4_GLNX86.mat")
    MAT73 = _p if os.path.exists(_p) else None
except ImportError:
    pass


@pytest.mark.skipif(MAT73 is None, reason="scipy's libhdf5-written test file is not installed")
def test_file_written_by_libhdf5(io, tmp_path):
    """scipy's test data holds an HDF5 file written by libhdf5 (MATLAB 7.4, 2008): a
    user block, superblock v0, the root group as a symbol table whose local heap has
    a free block, and the 1 x 9 double `testdouble` = 0, pi/4, ..., 2 pi."""
    got = io.read_hdf5(MAT73, "testdouble")
    assert got.dtype == np.float64 and got.size == 9
    assert np.allclose(got.ravel(), np.arange(9) * np.pi / 4)
    import shutil
    q = str(tmp_path / "copy.mat")
    shutil.copy(MAT73, q)
    io.write_hdf5(q, "CLUSTERS", np.arange(-4, 5))  # a new dataset in libhdf5's root group
    assert np.array_equal(io.read_hdf5(q, "testdouble"), got)
    assert np.array_equal(H.read_labels(q, "CLUSTERS"), np.arange(-4, 5))


# ------------------------------------------------------------------ errors of the reference

def test_missing_file(io, tmp_path):
    p = str(tmp_path / "none.h5")
    with pytest.raises(ValueError, match="^Could not open " + p + "$"):
        io.read_hdf5(p, "DATA")


@pytest.mark.parametrize("content", [b"", b"not an hdf5 file at all" * 10, H.SIG])
def test_not_hdf5(io, tmp_path, content):
    p = str(tmp_path / "bad.h5")
    with open(p, "wb") as fh:
        fh.write(content)
    with pytest.raises(ValueError, match="^Could not open "):
        io.read_hdf5(p, "DATA")


def test_directory_is_not_a_file(io, tmp_path):
    with pytest.raises(ValueError, match="^Could not open "):
        io.read_hdf5(str(tmp_path), "DATA")


@pytest.mark.parametrize("shape", [(10,), (2, 3, 4)])
def test_not_a_matrix(io, tmp_path, shape):
    p = str(tmp_path / "x.h5")
    H.write_matrix(p, np.zeros(shape, np.float32))
    with pytest.raises(ValueError, match="^Data in dataset DATA should be a matrix$"):
        io.read_hdf5(p, "DATA")


@pytest.mark.parametrize("msg,expect", [
    (H.dt_fixed(3, True, precision=24), "Unsupported signed integer precision"),
    (H.dt_fixed(3, False, precision=24), "Unsupported unsigned integer precision"),
    (H.dt_float(2), "Unsupported floating point precision"),
    (H.dt_string(4), "Unsupported data set type"),
])
def test_unsupported_element_types(io, tmp_path, msg, expect):
    p = str(tmp_path / "x.h5")
    H.write_matrix(p, np.zeros((4, 3), np.uint8), dtype_msg=msg)
    with pytest.raises(ValueError, match="^" + expect + "$"):
        io.read_hdf5(p, "DATA")


def test_filtered_storage_is_a_read_failure(io, tmp_path):
    p = str(tmp_path / "x.h5")
    deflate = bytes([1, 1, 0, 0, 0, 0, 0, 0]) + bytes([1, 0, 0, 0, 1, 0, 1, 0]) + (6).to_bytes(4, "little") + b"\0" * 4
    H.write_matrix(p, _points(np.float32), layout="chunked", chunk=(8, 3), extra=[(0x0B, 0, deflate)])
    with pytest.raises(RuntimeError, match=r"^Failed to read data \(filtered or compressed datasets\)$"):
        io.read_hdf5(p, "DATA")


def test_truncated_file(io, tmp_path):
    p = str(tmp_path / "x.h5")
    H.write_matrix(p, _points(np.float64, n=300))
    raw = open(p, "rb").read()
    with open(p, "wb") as fh:
        fh.write(raw[:len(raw) - 100])
    with pytest.raises(ValueError, match=r"^Could not open " + p + r" \(truncated file\)$"):
        io.read_hdf5(p, "DATA")
    # a dataset whose storage lies past the end of the file
    H.write_matrix(p, _points(np.float64, n=300))
    raw = bytearray(open(p, "rb").read())
    raw[40:48] = (len(raw) - 1000).to_bytes(8, "little")  # end-of-file address before the data's end
    with open(p, "wb") as fh:
        fh.write(raw[:len(raw) - 1000])
    with pytest.raises((ValueError, RuntimeError), match="address out of the file"):
        io.read_hdf5(p, "DATA")


# ------------------------------------------------------------------ writing labels

def test_write_new_file(io, tmp_path):
    p = str(tmp_path / "out.h5")
    labels = np.array([-1, -1, 2, 0, -5, 5, 0], np.int64)
    io.write_hdf5(p, "CLUSTERS", labels)
    got = H.check_structure(p, ["CLUSTERS"])
    assert np.array_equal(got["CLUSTERS"], labels)


def test_write_empty_labels(io, tmp_path):
    p = str(tmp_path / "out.h5")
    io.write_hdf5(p, "CLUSTERS", np.zeros(0, np.int64))
    assert H.read_labels(p, "CLUSTERS").size == 0


def test_write_into_the_input_file(io, tmp_path):
    """The reference CLI's default: -i data.h5 -o data.h5, labels added beside DATA."""
    p = str(tmp_path / "data.h5")
    pts = _points(np.float32, n=100)
    H.write_matrix(p, pts)
    labels = np.arange(-50, 50, dtype=np.int64)
    io.write_hdf5(p, "CLUSTERS", labels)
    assert np.array_equal(io.read_hdf5(p, "DATA"), pts)
    assert np.array_equal(H.read_labels(p, "CLUSTERS"), labels)
    again = labels[::-1].copy()
    io.write_hdf5(p, "CLUSTERS", again)  # existing dataset: overwritten in place
    assert np.array_equal(H.read_labels(p, "CLUSTERS"), again)
    assert np.array_equal(io.read_hdf5(p, "DATA"), pts)


def test_write_many_datasets_splits_symbol_table_nodes(io, tmp_path):
    p = str(tmp_path / "many.h5")
    expect = {}
    rng = np.random.default_rng(3)
    for i in rng.permutation(60):
        nm = f"L{i:02d}"
        expect[nm] = rng.integers(-1000, 1000, size=int(i) + 1)
        io.write_hdf5(p, nm, expect[nm])
    got = H.check_structure(p, sorted(expect))
    for nm, v in expect.items():
        assert np.array_equal(got[nm], v)


def test_write_into_a_file_with_a_two_level_group_tree_adds_nothing_silently(io, tmp_path):
    f = H.H5("earliest")
    kids = {f"set{i:03d}": f.dataset(_points(np.float32, n=4, seed=i)) for i in range(40)}
    p = str(tmp_path / "many.h5")
    f.finish(kids, p, levels=2)
    with pytest.raises(ValueError, match=r"^Could not open dataset NEW \(adding to a group B-tree of more than one level\)$"):
        io.write_hdf5(p, "NEW", np.arange(3))
    # an existing dataset of such a file is still written (a 2-D one of exactly n elements)
    io.write_hdf5(p, "set005", np.arange(12))
    assert np.array_equal(io.read_hdf5(p, "set005"), np.arange(12, dtype=np.float32).reshape(4, 3))


def test_write_nested_dataset(io, tmp_path):
    p = str(tmp_path / "x.h5")
    H.write_matrix(p, _points(np.float32), name="grp/DATA")
    io.write_hdf5(p, "grp/CLUSTERS", np.arange(7))
    assert np.array_equal(io.read_hdf5(p, "grp/DATA"), _points(np.float32))
    with pytest.raises(ValueError, match="^Could not open dataset nogroup/CLUSTERS$"):
        io.write_hdf5(p, "nogroup/CLUSTERS", np.arange(7))


@pytest.mark.parametrize("dt,expect", [
    (np.int32, [-2147483648, -1, 0, 7, 2147483647]),
    (np.uint8, [0, 0, 0, 7, 255]),
    (np.int64, [-(1 << 40), -1, 0, 7, 1 << 40]),
    (np.float64, [-(1 << 40), -1, 0, 7, 1 << 40]),
])
def test_write_converts_into_existing_element_types(io, tmp_path, dt, expect):
    """H5Dwrite of H5T_NATIVE_LONG into another type: integers saturate, floats round."""
    p = str(tmp_path / "x.h5")
    f = H.H5("earliest")
    f.finish({"CLUSTERS": f.dataset(np.zeros((5, 1), dt))}, p)
    io.write_hdf5(p, "CLUSTERS", np.array([-(1 << 40), -1, 0, 7, 1 << 40]))
    got = io.read_hdf5(p, "CLUSTERS")[:, 0]
    assert np.array_equal(got, np.array(expect, dtype=dt))


def test_write_first_elements_of_a_longer_dataset(io, tmp_path):
    p = str(tmp_path / "x.h5")
    io.write_hdf5(p, "CLUSTERS", np.full(10, 9))
    io.write_hdf5(p, "CLUSTERS", np.arange(4))
    assert np.array_equal(H.read_labels(p, "CLUSTERS"), [0, 1, 2, 3, 9, 9, 9, 9, 9, 9])


def test_write_wrong_size(io, tmp_path):
    p = str(tmp_path / "x.h5")
    io.write_hdf5(p, "CLUSTERS", np.arange(4))
    with pytest.raises(RuntimeError, match="^Failed to write data, target data set is probably of wrong size or type"):
        io.write_hdf5(p, "CLUSTERS", np.arange(5))
    assert np.array_equal(H.read_labels(p, "CLUSTERS"), np.arange(4))


def test_write_into_unwritten_storage(io, tmp_path):
    p = str(tmp_path / "x.h5")
    f = H.H5("earliest")
    f.finish({"CLUSTERS": f.dataset(np.zeros((6, 1), np.int64), unwritten=True, fill=np.int64(-3).tobytes())}, p)
    io.write_hdf5(p, "CLUSTERS", np.arange(6))
    assert np.array_equal(io.read_hdf5(p, "CLUSTERS")[:, 0], np.arange(6))


def test_write_latest_format(io, tmp_path):
    p = str(tmp_path / "x.h5")
    f = H.H5("latest")
    f.finish({"DATA": f.dataset(_points(np.float32)), "CLUSTERS": f.dataset(np.zeros((57, 1), np.int64))}, p)
    io.write_hdf5(p, "CLUSTERS", np.arange(57))  # existing contiguous dataset: in place
    assert np.array_equal(io.read_hdf5(p, "CLUSTERS")[:, 0], np.arange(57))
    with pytest.raises(ValueError, match=r"^Could not open dataset NEW \("):
        io.write_hdf5(p, "NEW", np.arange(57))


def test_write_errors(io, tmp_path):
    p = str(tmp_path / "not.h5")
    with open(p, "wb") as fh:
        fh.write(b"plain text")
    with pytest.raises(ValueError, match="^Could not open " + p + "$"):
        io.write_hdf5(p, "CLUSTERS", np.arange(3))
    with pytest.raises(ValueError, match="^Could not open "):
        io.write_hdf5(str(tmp_path / "missing_dir" / "x.h5"), "CLUSTERS", np.arange(3))
    q = str(tmp_path / "x.h5")
    H.write_matrix(q, _points(np.float32), name="grp/DATA")
    with pytest.raises(ValueError, match="^Could not open dataset grp$"):
        io.write_hdf5(q, "grp", np.arange(3))  # a group of that name
    assert not os.path.exists(str(tmp_path / "missing_dir"))


def test_lookup3_known_answers():
    """The test files' checksum: Bob Jenkins' published hashlittle values."""
    assert H.lookup3(b"") == 0xDEADBEEF
    assert H.lookup3(b"Four score and seven years ago", 0) == 0x17770551
    assert H.lookup3(b"Four score and seven years ago", 1) == 0xCD628161


# ------------------------------------------------------------------ more of the format

def test_superblock_version_1(io, tmp_path):
    p = str(tmp_path / "x.h5")
    a = _points(np.float64)
    f = H.H5("earliest")
    f.finish({"DATA": f.dataset(a)}, p, sb_version=1)
    assert np.array_equal(io.read_hdf5(p, "DATA"), a)
    io.write_hdf5(p, "CLUSTERS", np.arange(57))  # the end-of-file field sits 4 bytes later
    assert np.array_equal(io.read_hdf5(p, "DATA"), a)
    raw = open(p, "rb").read()
    assert int.from_bytes(raw[44:52], "little") == len(raw)


@pytest.mark.parametrize("version", [1, 2])
@pytest.mark.parametrize("layout", ["contiguous", "compact", "chunked"])
def test_layout_message_versions_1_and_2(io, tmp_path, version, layout):
    p = str(tmp_path / "x.h5")
    a = _points(np.int32, n=23)
    H.write_matrix(p, a, layout=layout, chunk=(5, 2), layout_version=version)
    assert np.array_equal(io.read_hdf5(p, "DATA"), a)


@pytest.mark.parametrize("style", ["old", "v1"])
def test_fill_value_message_styles(io, tmp_path, style):
    p = str(tmp_path / "x.h5")
    H.write_matrix(p, np.zeros((4, 2), np.int16), unwritten=True, fill=np.int16(-9).tobytes(), fill_style=style)
    assert np.array_equal(io.read_hdf5(p, "DATA"), np.full((4, 2), -9, np.int16))


@pytest.mark.parametrize("hflags", [0x00, 0x01, 0x03, 0x06, 0x22, 0x12, 0x36])
def test_object_header_v2_variants(io, tmp_path, hflags):
    """Chunk-size fields of 1/2/4/8 bytes, stored times, attribute phase change values
    and per-message creation order, with and without a continuation block."""
    a = _points(np.float32, n=31)
    for split in (None, 2):
        p = str(tmp_path / "x.h5")
        H.write_matrix(p, a, fmt="latest", hflags=hflags, split=split)
        assert np.array_equal(io.read_hdf5(p, "DATA"), a)


@pytest.mark.parametrize("link_flags", [0x08, 0x04, 0x10, 0x1C])
def test_link_message_variants(io, tmp_path, link_flags):
    p = str(tmp_path / "x.h5")
    a = _points(np.uint8, n=12)
    f = H.H5("latest")
    kids = {"other": f.dataset(a[:3]), "DATA": f.dataset(a)}
    f.finish(kids, p, link_flags=link_flags)
    assert np.array_equal(io.read_hdf5(p, "DATA"), a)
    assert np.array_equal(io.read_hdf5(p, "other"), a[:3])


def test_dense_link_storage_is_reported(io, tmp_path):
    p = str(tmp_path / "x.h5")
    f = H.H5("latest")
    f.finish({"DATA": f.dataset(_points(np.float32))}, p, dense=True)
    with pytest.raises(ValueError, match=r"^Could not open dataset DATA \(groups with dense link storage\)$"):
        io.read_hdf5(p, "DATA")


def test_shared_datatype_is_reported(io, tmp_path):
    p = str(tmp_path / "x.h5")
    f = H.H5("earliest")
    a = np.zeros((3, 2), np.float32)
    shared = (0x03, 2, bytes([1, 0, 0, 0]) + H.q(4096))  # flag 2: the message points at a committed type
    hdr = f.header_v1([(0x01, 0, H.space_v1(a.shape)), shared, (0x05, 1, H.fill_v2()),
                       (0x08, 0, H.layout_contiguous(f.raw(a.tobytes()), a.nbytes))])
    f.finish({"DATA": hdr}, p)
    with pytest.raises(ValueError, match=r"^Could not open dataset DATA \(shared dataspace or datatype messages\)$"):
        io.read_hdf5(p, "DATA")


def test_write_into_compact_big_endian_and_chunked_targets(io, tmp_path):
    p = str(tmp_path / "x.h5")
    f = H.H5("earliest")
    kids = {"COMPACT": f.dataset(np.zeros((6, 1), np.int64), layout="compact"),
            "BIG": f.dataset(np.zeros((6, 1), np.int32), big=True),
            "CHUNKED": f.dataset(np.zeros((6, 1), np.int64), layout="chunked", chunk=(4, 1))}
    f.finish(kids, p)
    io.write_hdf5(p, "COMPACT", np.arange(6) - 3)
    assert np.array_equal(io.read_hdf5(p, "COMPACT")[:, 0], np.arange(6) - 3)
    io.write_hdf5(p, "BIG", np.array([-5, 70000, 3, 1 << 40, -(1 << 40), 0]))
    assert np.array_equal(io.read_hdf5(p, "BIG")[:, 0], [-5, 70000, 3, 2**31 - 1, -2**31, 0])
    with pytest.raises(RuntimeError, match=r"\(writing chunked datasets\)$"):
        io.write_hdf5(p, "CHUNKED", np.arange(6))
    q = str(tmp_path / "latest.h5")
    g = H.H5("latest")
    g.finish({"COMPACT": g.dataset(np.zeros((6, 1), np.int64), layout="compact")}, q)
    with pytest.raises(RuntimeError, match=r"\(compact data inside a checksummed object header\)$"):
        io.write_hdf5(q, "COMPACT", np.arange(6))
