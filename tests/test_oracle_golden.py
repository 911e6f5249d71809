"""The oracle against the golden vectors produced by the reference's own host
code (tests/golden/make_golden.py): the REF16 mode must reproduce them bit for
bit on x86-64 (where they were generated), and within float rounding elsewhere."""
import platform

import numpy as np
import pytest

from conftest import golden_fields, map_errors

X86 = platform.machine() in ("x86_64", "AMD64")


def _case_args(meta, case):
    c = meta["cases"][case]
    nside, steps, batch = c["nside"], c["n_steps"], c["batch"]
    begin, count = (0, 12 * nside * nside) if batch is None else (batch * nside * nside, nside * nside)
    return nside, steps, begin, count


@pytest.mark.parametrize("case", ["cube16_ns2_s12", "cube32_ns4_s24", "cube24_ns3_s20", "wrap16_ns2_s40",
                                  "batch5_cube32_ns4_s16", "noncubic_16x20x24_ns2_s14", "zero16_ns2_s10"])
def test_ref16_oracle_matches_reference_bits(golden, orc, case):
    meta, maps = golden
    phi, b = golden_fields(meta, case)
    nside, steps, begin, count = _case_args(meta, case)
    got = orc.trace(phi, b, nside, steps, begin, count, mode="ref16")
    want = maps[case][:, begin:begin + count]
    if X86:
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), case
    else:
        for rms, mx in map_errors(got, want):
            assert rms < 1e-5 and mx < 1e-3
    # outside the batch range the reference's maps are exactly zero (snapshot-raytracer.cu:932-942)
    outside = np.ones(maps[case].shape[1], bool)
    outside[begin:begin + count] = False
    assert not np.any(maps[case][:, outside])


@pytest.mark.parametrize("case", ["cube16_ns2_s12", "cube32_ns4_s24", "wrap16_ns2_s40",
                                  "noncubic_16x20x24_ns2_s14"])
def test_fp64_oracle_close_to_reference(golden, orc, case):
    """FP64 restatement vs the reference's FP16/FP32 arithmetic: the difference
    is the reference's own rounding (B quantised to 11 bits, FP32 offsets)."""
    meta, maps = golden
    phi, b = golden_fields(meta, case)
    nside, steps, begin, count = _case_args(meta, case)
    got = orc.trace(phi, b, nside, steps, begin, count, mode="fp64")
    for m, (rms, mx) in enumerate(map_errors(got, maps[case][:, begin:begin + count])):
        assert rms < 1e-4, (m, rms)
        assert mx < 1e-3, (m, mx)


def test_zero_fields_exact(golden, orc):
    """Phi = B = 0: straight rays; dA' = -1 so dA = n_steps exactly, no shear,
    no rotation, deflection zero to rounding (snapshot-raytracer.cu:481-509)."""
    meta, maps = golden
    case = "zero16_ns2_s10"
    steps = meta["cases"][case]["n_steps"]
    m = maps[case]
    assert np.all(m[0] == steps)
    assert not np.any(m[1:4])
    assert np.abs(m[4:6]).max() < 1e-12
    phi, b = golden_fields(meta, case)
    got = orc.trace(phi, b, 2, steps, mode="fp64")
    assert np.all(got[0] == steps) and not np.any(got[1:4])


def test_interpolation_matches_reference(golden, orc):
    meta, maps = golden
    want = maps["interp"]
    for i, (case, f, x, y, z) in enumerate(meta["interp_points"]):
        phi, b = golden_fields(meta, case)
        got = orc.interp(phi, b, f, x, y, z, mode="ref16")
        if X86:
            assert np.array_equal(got, want[i]), (case, f, x, y, z)
        else:
            np.testing.assert_allclose(got, want[i], rtol=1e-5, atol=1e-12)
        g64 = orc.interp(phi, b, f, x, y, z, mode="fp64")
        scale = np.abs(want[i]).max() + 1e-30
        assert np.abs(g64 - want[i]).max() < 2e-3 * scale


def test_half_conversion_round_to_nearest_even(orc):
    """The oracle's float -> binary16 conversion (vector3_to_half's
    __float2half, snapshot-raytracer.cu:589) against numpy's IEEE conversion."""
    rng = np.random.default_rng(0)
    vals = np.concatenate([rng.standard_normal(20000).astype(np.float32) * np.float32(s)
                           for s in (1e-8, 1e-5, 1e-2, 1.0, 13.0, 1e3, 6e4)])
    specials = np.array([0.0, -0.0, 65504.0, 65519.0, 65520.0, 1e9, -1e9, 2.0 ** -24, 2.0 ** -25,
                         1.5 * 2.0 ** -25, 2.0 ** -14, np.inf, -np.inf], np.float32)
    for v in np.concatenate([vals, specials]):
        got = orc.float_to_half_bits(v)
        with np.errstate(over="ignore"):  # values beyond the half range become inf, as intended
            want = int(np.array(v, np.float32).astype(np.float16).view(np.uint16))
        assert got == want, (v, hex(got), hex(want))
        assert orc.half_bits_to_float(want) == float(np.array(want, np.uint16).view(np.float16))


@pytest.mark.skipif("not __import__('oracle.oracle', fromlist=['x']).ref_available()")
def test_ref16_oracle_matches_reference_on_gaussian_fields(orc):
    """Where the reference sources exist: the port against the reference's own
    host code on a Gaussian field (not only the integer fixtures)."""
    import srt_fields

    phi, b = srt_fields.gaussian_fields_np(32, seed=11)
    got = orc.trace(phi, b, 4, 20, mode="ref16")
    want = orc.ref_trace(phi, b, 4, 20)
    if X86:
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_constant_gradient_potential_analytic(orc):
    """FP64 oracle against the first-order analytic deflection and dA of a
    constant-gradient potential."""
    from conftest import check_linear_phi_maps, linear_phi_case

    phi, b, predict = linear_phi_case()
    nside, S = 2, 20
    maps = orc.trace(phi, b, nside, S, mode="fp64")
    check_linear_phi_maps(maps, nside, S, predict, orc.pix2ang_ring)
