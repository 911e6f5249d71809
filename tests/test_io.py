"""Host file formats of the CLI contract (no GPU): HDF5 /data datasets in and
HEALPix FITS maps out (snapshot-raytracer.cu:22-186, :941-987)."""
import os
import struct
import subprocess

import numpy as np
import pytest

from conftest import PKG

CLI = os.path.join(PKG, "snapshot-raytracer")


@pytest.mark.parametrize("shape", [(5,), (4, 6), (3, 4, 5), (2, 3, 4, 5)])
def test_h5_scalar_roundtrip(srt, tmp_path, shape):
    a = np.random.default_rng(1).standard_normal(shape).astype(np.float32)
    p = str(tmp_path / "s.h5")
    srt.h5_write(p, a)
    b = srt.h5_read_scalar(p)
    assert b.shape == shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_h5_vector3_roundtrip_and_type_checks(srt, tmp_path):
    v = np.random.default_rng(2).standard_normal((4, 5, 6, 3)).astype(np.float32)
    p = str(tmp_path / "v.h5")
    srt.h5_write(p, v, vector3=True)
    w = srt.h5_read_vector3(p)
    assert w.shape == v.shape and np.array_equal(v, w)
    # the reference's checks (snapshot-raytracer.cu:113-143): B must be rank 3
    # with an array[3] element type; a scalar dataset is refused
    s = str(tmp_path / "s.h5")
    srt.h5_write(s, v[..., 0])
    with pytest.raises(srt.SrtError, match="not an array type"):
        srt.h5_read_vector3(s)
    with pytest.raises(srt.SrtError, match="array element type"):
        srt.h5_read_scalar(p)


def test_h5_errors(srt, tmp_path):
    with pytest.raises(srt.SrtError, match="Failed to open HDF5 file"):
        srt.h5_read_scalar(str(tmp_path / "missing.h5"))
    bad = tmp_path / "bad.h5"
    bad.write_bytes(b"not hdf5" * 100)
    with pytest.raises(srt.SrtError, match="not an HDF5 file"):
        srt.h5_read_scalar(str(bad))
    p = str(tmp_path / "s.h5")
    srt.h5_write(p, np.zeros((2, 2, 2), np.float32))
    with pytest.raises(srt.SrtError, match="no object"):
        srt.h5_read_scalar(p, "/other")
    # truncated file
    raw = open(p, "rb").read()
    t = tmp_path / "trunc.h5"
    t.write_bytes(raw[: len(raw) - 16])
    with pytest.raises(srt.SrtError):
        srt.h5_read_scalar(str(t))


def test_h5_file_structure(srt, tmp_path):
    """The writer's layout: superblock v0 at byte 0 with 8-byte offsets, the
    raw little-endian floats at the end of the file."""
    a = np.arange(24, dtype=np.float32).reshape(2, 3, 4)
    p = str(tmp_path / "s.h5")
    srt.h5_write(p, a)
    raw = open(p, "rb").read()
    assert raw[:8] == b"\x89HDF\r\n\x1a\n" and raw[8] == 0 and raw[13] == 8 and raw[14] == 8
    assert raw[-96:] == a.tobytes()
    eof = struct.unpack("<Q", raw[40:48])[0]
    assert eof == len(raw)


@pytest.mark.parametrize("nest", [False, True])
def test_fits_roundtrip(srt, tmp_path, nest):
    nside = 4
    m = np.random.default_rng(3).standard_normal(12 * nside * nside).astype(np.float32)
    p = str(tmp_path / "m.fits")
    srt.fits_write_map(p, m, nside, nest=nest)
    got, ns, ne = srt.fits_read_map(p)
    assert ns == nside and ne == nest and np.array_equal(got, m)
    raw = open(p, "rb").read()
    assert len(raw) % 2880 == 0
    assert raw[:30] == b"SIMPLE  =                    T"
    hdr = raw[2880:2880 * 2].decode("ascii")
    assert "XTENSION= 'BINTABLE'" in hdr and "TFORM1  = '1E      '" in hdr
    assert ("ORDERING= '%s" % ("NESTED" if nest else "RING")) in hdr and "COORDSYS= 'C       '" in hdr
    # big-endian float32 rows start after the extension header
    assert struct.unpack(">f", raw[2 * 2880:2 * 2880 + 4])[0] == m[0]


def test_fits_does_not_overwrite_by_default(srt, tmp_path):
    p = str(tmp_path / "m.fits")
    srt.fits_write_map(p, np.zeros(12, np.float32), 1)
    with pytest.raises(srt.SrtError, match="already exists"):
        srt.fits_write_map(p, np.ones(12, np.float32), 1)
    srt.fits_write_map(p, np.ones(12, np.float32), 1, overwrite=True)
    assert np.all(srt.fits_read_map(p)[0] == 1)


def run_cli(*args, cwd=None):
    return subprocess.run([CLI, *map(str, args)], capture_output=True, text=True, cwd=cwd)


def test_cli_usage_and_argument_errors(tmp_path):
    """snapshot-raytracer.cu:602-631: usage on stderr and status 255 (return -1)."""
    r = run_cli()
    assert r.returncode == 255 and r.stderr.startswith("Usage: ") and "<hdf5_file_potential>" in r.stderr
    r = run_cli("a.h5", "b.h5", "0", "10")
    assert r.returncode == 255 and "Invalid Nside value: 0" in r.stderr
    r = run_cli("a.h5", "b.h5", "4", "-3")
    assert r.returncode == 255 and "Invalid n_steps value: -3" in r.stderr
    r = run_cli("a.h5", "b.h5", "4", "10", "-1")
    assert r.returncode == 255 and "Invalid batch value: -1" in r.stderr
    r = run_cli("a.h5", "b.h5", "four", "10")
    assert r.returncode == 255 and "Invalid Nside value" in r.stderr
    for bad in ("abc", "inf", "nan", "2x"):
        r = run_cli("a.h5", "b.h5", "4", "10", "--rescale-phi", bad)
        assert r.returncode == 255 and "Invalid rescaling factor: %s" % bad in r.stderr
    r = run_cli("a.h5", "b.h5", "4", "10", "--rescale-b", "")
    assert r.returncode == 255 and "Invalid rescaling factor" in r.stderr
    r = run_cli(tmp_path / "missing.h5", "b.h5", "4", "10")
    assert r.returncode == 255
    assert r.stdout.splitlines()[:3] == ["Nside: 4", "n_steps: 10",
                                         "Loading potential data from HDF5 file %s ..." % (tmp_path / "missing.h5")]
    assert "Failed to open HDF5 file" in r.stderr


def test_cli_rejects_bad_b_and_batch(srt, tmp_path):
    import srt_fields

    phi, b = srt_fields.int_noise_fields(8, seed=1)
    pp, pb, pb2 = str(tmp_path / "phi.h5"), str(tmp_path / "b.h5"), str(tmp_path / "b2.h5")
    srt.h5_write(pp, phi)
    srt.h5_write(pb, b, vector3=True)
    srt.h5_write(pb2, b[..., 0])  # not array[3]
    r = run_cli(pp, pb2, 2, 4)
    assert r.returncode == 255 and "not an array type" in r.stderr
    r = run_cli(pp, pb, 2, 4, 12)
    assert r.returncode == 255 and "Batch exceeds total number of pixels" in r.stderr
    small = str(tmp_path / "bs.h5")
    srt.h5_write(small, b[:4], vector3=True)
    r = run_cli(pp, small, 2, 4)
    assert r.returncode == 255 and "differ" in r.stderr


@pytest.mark.parametrize("dtype", ["<f4", ">f8", "<f8", ">i2", "<u1"])
@pytest.mark.parametrize("filters", [(), ("deflate",), ("shuffle", "deflate")])
def test_h5_reader_v2_chunked_variants(srt, tmp_path, dtype, filters):
    import h5_variants

    rng = np.random.default_rng(4)
    a = (rng.standard_normal((7, 10, 9)) * (1 if np.dtype(dtype).kind == "f" else 20)).astype(dtype)
    if np.dtype(dtype).kind == "u":
        a = np.abs(a)
    p = str(tmp_path / "v2.h5")
    h5_variants.write_v2_chunked(p, a, chunk=(3, 4, 5), filters=filters)
    got = srt.h5_read_scalar(p)
    assert got.shape == a.shape
    assert np.array_equal(got, a.astype(np.float64).astype(np.float32))


def test_h5_reader_many_chunks_in_parallel_and_a_corrupt_chunk(srt, tmp_path):
    """528 deflated chunks read and unfiltered on all host threads land in the
    right places; a corrupt chunk in the middle is reported from whichever
    thread met it, as an error status with a message."""
    import h5_variants

    a = np.random.default_rng(6).standard_normal((40, 36, 44)).astype(np.float32)
    p = str(tmp_path / "many.h5")
    h5_variants.write_v2_chunked(p, a, chunk=(5, 6, 4))
    assert np.array_equal(srt.h5_read_scalar(p), a)
    raw = bytearray(open(p, "rb").read())
    mid = len(raw) // 3  # inside the chunk data, which follows the 48-byte superblock
    raw[mid:mid + 64] = bytes(64)
    q = str(tmp_path / "corrupt.h5")
    open(q, "wb").write(bytes(raw))
    with pytest.raises(srt.SrtError) as ei:
        srt.h5_read_scalar(q)
    assert "corrupt deflate chunk" in str(ei.value)


def test_h5_reader_chunk_size_past_end_of_file(srt, tmp_path):
    """A chunk whose stored size (a 32-bit field of its B-tree entry) is
    corrupt and reaches past the end of the file is refused with a format
    error before anything is allocated for it, whichever thread reads it."""
    import struct

    import h5_variants

    a = np.random.default_rng(7).standard_normal((20, 18, 22)).astype(np.float32)
    p = str(tmp_path / "ok.h5")
    h5_variants.write_v2_chunked(p, a, chunk=(5, 6, 4))
    raw = bytearray(open(p, "rb").read())
    at = raw.index(b"TREE" + bytes([1, 0]))  # first leaf node
    entry = at + 8 + 16                      # after signature, type, level, count and two sibling addresses
    raw[entry:entry + 4] = struct.pack("<I", 0xFFFFFF00)
    q = str(tmp_path / "huge_chunk.h5")
    open(q, "wb").write(bytes(raw))
    with pytest.raises(srt.SrtError) as ei:
        srt.h5_read_scalar(q)
    assert ei.value.code == -5 and "past the end" in str(ei.value)


@pytest.mark.parametrize("fanout", [64, 3])
def test_h5_reader_multilevel_chunk_btree(srt, tmp_path, fanout):
    """Chunk B-trees of several levels, as libhdf5 writes them for many chunks
    (2K = 64 entries per node; fanout 3 gives five levels here)."""
    import h5_variants

    a = np.random.default_rng(8).standard_normal((24, 20, 28)).astype(np.float32)
    p = str(tmp_path / ("ml%d.h5" % fanout))
    h5_variants.write_v2_chunked(p, a, chunk=(4, 4, 4), fanout=fanout)  # 6 x 5 x 7 = 210 chunks
    assert np.array_equal(srt.h5_read_scalar(p), a)
    v = np.random.default_rng(9).standard_normal((9, 8, 10, 3)).astype(np.float32)
    q = str(tmp_path / ("mlv%d.h5" % fanout))
    h5_variants.write_v2_chunked(q, v, chunk=(2, 3, 4), array3=True, fanout=fanout)
    assert np.array_equal(srt.h5_read_vector3(q), v)


def test_h5_reader_vector3_chunked(srt, tmp_path):
    import h5_variants

    v = np.random.default_rng(5).standard_normal((5, 6, 7, 3)).astype(np.float32)
    p = str(tmp_path / "vc.h5")
    h5_variants.write_v2_chunked(p, v, chunk=(2, 3, 7), array3=True)
    assert np.array_equal(srt.h5_read_vector3(p), v)


def test_h5_reader_v0_continuation(srt, tmp_path):
    import h5_variants

    a = np.random.default_rng(6).standard_normal((4, 5, 6)).astype(">f4")
    p = str(tmp_path / "v0c.h5")
    h5_variants.write_v0_continuation(p, a)
    assert np.array_equal(srt.h5_read_scalar(p), a.astype(np.float32))
