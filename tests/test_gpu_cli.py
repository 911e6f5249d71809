"""The CLI drop-in end to end on the GPU: HDF5 inputs -> six FITS maps with the
reference's names, RING order, batch masking and stdout progress lines
(snapshot-raytracer.cu:600-1007)."""
import os
import subprocess

import numpy as np
import pytest

import srt_fields
from conftest import PKG, golden_fields, map_errors

pytestmark = pytest.mark.gpu
CLI = os.path.join(PKG, "snapshot-raytracer")
NAMES = ["dAmap", "ellipticity1map", "ellipticity2map", "rotationmap", "deflection1map", "deflection2map"]
STDOUT = ["Nside: {nside}", "n_steps: {steps}", "Loading potential data from HDF5 file {phi} ...",
          "Data dimensions: {d0} x {d1} x {d2}", "Loading B field data from HDF5 file {b} ...",
          "Allocating device memory and copying data to device...", "Computing theta and phi angles...",
          "Launching raytracing kernel...", "Raytracing completed.", "Saving results to FITS files...", "All done!"]


def write_inputs(srt, tmp_path, phi, b):
    pp, pb = str(tmp_path / "phi.h5"), str(tmp_path / "B.h5")
    # HDF5 dims in file order; the reference takes dims[0] as the fastest extent
    srt.h5_write(pp, phi)
    srt.h5_write(pb, b, vector3=True)
    return pp, pb


@pytest.mark.parametrize("batch", [None, 3])
def test_cli_maps_match_library(srt, tmp_path, batch):
    phi, b = srt_fields.gaussian_fields_np(32, seed=5)
    pp, pb = write_inputs(srt, tmp_path, phi, b)
    nside, steps = 4, 16
    args = [CLI, pp, pb, str(nside), str(steps)] + ([] if batch is None else [str(batch)])
    r = subprocess.run(args, capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    want_out = [s.format(nside=nside, steps=steps, phi=pp, b=pb, d0=32, d1=32, d2=32) for s in STDOUT]
    assert r.stdout.splitlines() == want_out
    ref = srt.trace(phi, b, nside, steps, batch=batch, precision="mixed")
    for m, name in enumerate(NAMES):
        got, ns, nest = srt.fits_read_map(str(tmp_path / ("%s_batch%d.fits" % (name, 0 if batch is None else batch))))
        assert ns == nside and not nest
        assert np.array_equal(got.view(np.uint32), ref[m].view(np.uint32)), name


def test_cli_rescale_options(srt, tmp_path):
    """--rescale-phi / --rescale-b: the runtime form of the reference's
    RESCALE_DATA / RESCALE_BDATA (snapshot-raytracer.cu:663-670, :681-688),
    with its messages after each field is loaded."""
    phi, b = srt_fields.gaussian_fields_np(24, seed=7)
    pp, pb = write_inputs(srt, tmp_path, phi, b)
    nside, steps = 4, 12
    r = subprocess.run([CLI, pp, pb, str(nside), str(steps), "--precision", "fp64", "--rescale-phi", "2",
                        "--rescale-b", "0.25"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    assert lines[3:7] == ["Data dimensions: 24 x 24 x 24", "Rescaling potential data by factor 2",
                          "Loading B field data from HDF5 file %s ..." % pb, "Rescaling B field data by factor 0.25"]
    ref = srt.trace((phi.astype(np.float64) * 2).astype(np.float32), (b.astype(np.float64) * 0.25).astype(np.float32),
                    nside, steps, precision="fp64")
    for m, name in enumerate(NAMES):
        got = srt.fits_read_map(str(tmp_path / ("%s_batch0.fits" % name)))[0]
        assert np.array_equal(got.view(np.uint32), ref[m].view(np.uint32)), name


def test_cli_ref16_reproduces_reference_golden(srt, golden, tmp_path):
    meta, maps = golden
    case = "batch5_cube32_ns4_s16"
    phi, b = golden_fields(meta, case)
    pp, pb = write_inputs(srt, tmp_path, phi, b)
    c = meta["cases"][case]
    r = subprocess.run([CLI, pp, pb, str(c["nside"]), str(c["n_steps"]), str(c["batch"]), "--precision", "ref16"],
                       capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    got = np.stack([srt.fits_read_map(str(tmp_path / ("%s_batch%d.fits" % (n, c["batch"]))))[0] for n in NAMES])
    want = maps[case]
    outside = np.ones(want.shape[1], bool)
    lo = c["batch"] * c["nside"] ** 2
    outside[lo:lo + c["nside"] ** 2] = False
    assert not np.any(got[:, outside])
    for rms, mx in map_errors(got[:, ~outside], want[:, ~outside]):
        assert rms < 1e-5 and mx < 2e-3


def test_cli_keeps_existing_outputs(srt, tmp_path):
    phi, b = srt_fields.int_noise_fields(16, seed=8)
    pp, pb = write_inputs(srt, tmp_path, phi, b)
    (tmp_path / "dAmap_batch0.fits").write_bytes(b"keep")
    r = subprocess.run([CLI, pp, pb, "2", "4"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0 and "already exists" in r.stderr
    assert (tmp_path / "dAmap_batch0.fits").read_bytes() == b"keep"
    r = subprocess.run([CLI, pp, pb, "2", "4", "--overwrite"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0
    assert srt.fits_read_map(str(tmp_path / "dAmap_batch0.fits"))[1] == 2


def test_cli_base_pixel_batch(srt, tmp_path):
    """--base-pixel: batch b is HEALPix base pixel b (NESTED range), the maps
    are zero outside it and equal the full-sky maps inside it."""
    phi, b = srt_fields.gaussian_fields_np(32, seed=6)
    pp, pb = write_inputs(srt, tmp_path, phi, b)
    nside, steps, face = 8, 16, 7
    r = subprocess.run([CLI, pp, pb, str(nside), str(steps), str(face), "--base-pixel"], capture_output=True,
                       text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    full = srt.trace(phi, b, nside, steps, precision="mixed")
    inside = np.zeros(12 * nside * nside, bool)
    inside[[srt.nest2ring(nside, face * nside * nside + i) for i in range(nside * nside)]] = True
    for m, name in enumerate(NAMES):
        got, ns, nest = srt.fits_read_map(str(tmp_path / ("%s_batch%d.fits" % (name, face))))
        assert ns == nside and not nest
        assert not np.any(got[~inside])
        assert np.array_equal(got[inside].view(np.uint32), full[m][inside].view(np.uint32)), name
    r = subprocess.run([CLI, pp, pb, "6", "4", "1", "--base-pixel"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 255 and "power-of-two" in r.stderr


def test_cli_hdf5_axis_order_noncubic(srt, tmp_path):
    """--xyz-order hdf5: x is the fastest HDF5 axis with its own extent, so a
    non-cubic grid gives the library's maps for the same array."""
    phi, b = srt_fields.gaussian_fields_np((24, 16, 20), seed=9)  # numpy shape (20, 16, 24): x extent 24
    pp, pb = write_inputs(srt, tmp_path, phi, b)
    nside, steps = 4, 12
    r = subprocess.run([CLI, pp, pb, str(nside), str(steps), "--xyz-order", "hdf5"], capture_output=True, text=True,
                       cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    ref = srt.trace(phi, b, nside, steps, precision="mixed")
    for m, name in enumerate(NAMES):
        got = srt.fits_read_map(str(tmp_path / ("%s_batch0.fits" % name)))[0]
        assert np.array_equal(got.view(np.uint32), ref[m].view(np.uint32)), name


@pytest.mark.parametrize("filters", [("shuffle", "deflate"), ("deflate",), ()], ids=["shuffle-deflate", "deflate",
                                                                                    "chunked"])
def test_cli_chunked_filtered_inputs_equal_contiguous(srt, tmp_path, filters):
    """Phi and B stored chunked (several chunks per axis, partial edge chunks,
    a chunk B-tree of several levels), with the shuffle and deflate filters as
    simulation snapshots are often written, traced through the CLI: the six
    FITS maps equal, bit for bit, those of the same fields stored contiguously
    (the reference reads either through libhdf5, snapshot-raytracer.cu:23-87,
    :92-186)."""
    import ctypes

    import h5_variants

    if "deflate" in filters:
        try:
            ctypes.CDLL("libz.so.1")
        except OSError:
            pytest.skip("the reader's deflate filter loads libz.so.1, absent here")
    phi, b = srt_fields.gaussian_fields_np(28, seed=12)
    nside, steps = 4, 14
    plain = tmp_path / "plain"
    chunked = tmp_path / "chunked"
    plain.mkdir()
    chunked.mkdir()
    pp, pb = write_inputs(srt, plain, phi, b)
    cp, cb = str(chunked / "phi.h5"), str(chunked / "B.h5")
    h5_variants.write_v2_chunked(cp, phi, chunk=(8, 6, 10), filters=filters, fanout=5)
    h5_variants.write_v2_chunked(cb, b, chunk=(5, 9, 7), filters=filters, array3=True, fanout=4)
    for d, (p1, p2) in ((plain, (pp, pb)), (chunked, (cp, cb))):
        r = subprocess.run([CLI, p1, p2, str(nside), str(steps), "2"], capture_output=True, text=True, cwd=d)
        assert r.returncode == 0, r.stderr
    for name in NAMES:
        want = srt.fits_read_map(str(plain / ("%s_batch2.fits" % name)))[0]
        got = srt.fits_read_map(str(chunked / ("%s_batch2.fits" % name)))[0]
        assert np.any(want) and np.array_equal(got.view(np.uint32), want.view(np.uint32)), name


@pytest.mark.parametrize("layout", ["contiguous", "chunked", "hdf5-order"])
def test_fields_load_h5_equals_host_arrays(srt, tmp_path, layout):
    """srt_fields_load_h5 reads the two files on a reader thread while every
    finished run of planes is copied and laid out on the device: the handle
    traces exactly as one made by srt_fields_create from the same arrays
    (contiguous and chunked/deflated files, rescaled values, the HDF5 axis
    order of a non-cubic grid), and its statistics account for the bytes."""
    import ctypes

    import h5_variants

    shape = (20, 24, 28) if layout == "hdf5-order" else (24, 24, 24)
    phi, b = srt_fields.gaussian_fields_np(shape, seed=14)  # numpy shape (n2, n1, n0)
    pp, pb = str(tmp_path / "phi.h5"), str(tmp_path / "B.h5")
    if layout == "chunked":
        try:
            ctypes.CDLL("libz.so.1")
            filters = ("shuffle", "deflate")
        except OSError:
            filters = ()
        h5_variants.write_v2_chunked(pp, phi, chunk=(5, 7, 6), filters=filters, fanout=3)
        h5_variants.write_v2_chunked(pb, b, chunk=(4, 6, 9), filters=filters, array3=True)
    else:
        srt.h5_write(pp, phi)
        srt.h5_write(pb, b, vector3=True)
    nside, steps = 4, 12
    f, st = srt.Fields.load_h5(pp, pb, xyz_order="hdf5" if layout == "hdf5-order" else "reference",
                               phi_scale=2.0, b_scale=0.5)
    with f:
        got, _ = f.forward(nside, steps, precision="fp64")
    phi2 = (phi.astype(np.float64) * 2.0).astype(np.float32)
    b2 = (b.astype(np.float64) * 0.5).astype(np.float32)
    if layout == "hdf5-order":
        with srt.Fields(phi2, b2) as g:  # (n2, n1, n0) = the file's shape, x fastest
            want, _ = g.forward(nside, steps, precision="fp64")
        assert st["n"] == (shape[0], shape[1], shape[2])
    else:
        with srt.Fields(phi2, b2) as g:
            want, _ = g.forward(nside, steps, precision="fp64")
        assert st["n"] == (24, 24, 24)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert st["h2d_bytes"] == 16 * phi.size and st["total_ms"] > 0 and st["read_phi_ms"] > 0
    # a B file whose extents differ from phi's is refused with the CLI's message
    q = str(tmp_path / "B_small.h5")
    srt.h5_write(q, np.zeros((4, 4, 4, 3), np.float32), vector3=True)
    with pytest.raises(srt.SrtError) as ei:
        srt.Fields.load_h5(pp, q)
    assert "differ from the potential's" in str(ei.value)
