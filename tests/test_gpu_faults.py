"""Failure injection on the GPU path without a GPU fault: device allocations
are made to fail one at a time through srt_debug_fail_alloc (the host-side
hook; nothing on the device misbehaves). The reference prints the failed
cudaMalloc and returns -1 (snapshot-raytracer.cu:752-772); here every call
that meets the failure must return SRT_ERR_OUT_OF_MEMORY with the name of the
allocation, release what it had allocated, and leave the library usable: the
next call without the failure gives the same result, bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SRT_ERR_OUT_OF_MEMORY = -3


def _sweep_failures(srt, call, max_allocs=64):
    """Runs call() with the hook armed after 0, 1, 2, ... allocations until a
    call completes; returns (number of failed calls, the completed result)."""
    L = srt.lib()
    failed = 0
    try:
        for after in range(max_allocs):
            assert L.srt_debug_fail_alloc(after) == 0
            try:
                out = call()
            except srt.SrtError as e:
                assert e.code == SRT_ERR_OUT_OF_MEMORY, str(e)
                assert "out of memory" in str(e)
                failed += 1
                continue
            finally:
                L.srt_debug_fail_alloc(-1)
            return failed, out
    finally:
        L.srt_debug_fail_alloc(-1)
    pytest.fail("a call made more than %d device allocations" % max_allocs)


def test_forward_allocation_failures(srt):
    import srt_fields

    phi, b = srt_fields.int_noise_fields(24, seed=5)
    nside, steps = 4, 16

    def forward():
        with srt.Fields(phi, b) as f:
            maps, _ = f.forward(nside, steps, precision="mixed")
        return maps

    want = forward()
    failed, got = _sweep_failures(srt, forward)
    # fields: phi, three B planes, the upload slab, four row-pair arrays;
    # forward: the re-trace list, its counter, the device maps
    assert failed >= 9
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(forward(), want)
    assert np.all(np.isfinite(want))


def test_vjp_allocation_failures(srt):
    import srt_fields

    phi, b = srt_fields.int_noise_fields(20, seed=6)
    nside, steps = 2, 12
    w = np.random.default_rng(7).standard_normal((6, 12 * nside * nside)).astype(np.float32)
    with srt.Fields(phi, b) as f:

        def vjp():
            gphi, gb, _ = f.vjp(nside, steps, w, precision="mixed", ckpt_every=4, deterministic=True)
            return gphi, gb

        want = vjp()
        failed, got = _sweep_failures(srt, vjp)
        again = vjp()
    # ray list and offsets, weights, checkpoints, tape, cotangents, accumulators
    assert failed >= 5
    for g, w_, a in zip(got, want, again):
        np.testing.assert_array_equal(g, w_)
        np.testing.assert_array_equal(a, w_)
        assert np.all(np.isfinite(w_))


def test_tape_pair_and_ref16_allocation_failures(srt):
    import srt_fields

    phi, b = srt_fields.int_noise_fields(20, seed=9)
    nside, steps = 2, 12
    w = np.random.default_rng(10).standard_normal((6, 12 * nside * nside)).astype(np.float32)
    with srt.Fields(phi, b) as f:

        def pair():
            maps, tape, _ = f.forward_tape(nside, steps, ckpt_every=4)
            try:
                gphi, gb, _ = tape.vjp(w, deterministic=True)
            finally:
                tape.close()
            return maps, gphi, gb

        want = pair()
        failed, got = _sweep_failures(srt, pair)
        # tape: rays, checkpoints, re-trace list and counter, maps; vjp: its buffers
        assert failed >= 5
        for g, w_ in zip(got, want):
            np.testing.assert_array_equal(g, w_)

    # REF16 makes its FP16 planes on first use: a failure there leaves the
    # handle usable and the next call makes them
    with srt.Fields(phi, b) as f:
        want16, _ = f.forward(nside, steps, precision="ref16")
    with srt.Fields(phi, b) as f:
        failed, got16 = _sweep_failures(srt, lambda: f.forward(nside, steps, precision="ref16")[0])
        assert failed >= 1
        np.testing.assert_array_equal(got16, want16)


def test_hook_disarms_itself(srt):
    import srt_fields

    phi, b = srt_fields.int_noise_fields(16, seed=8)
    L = srt.lib()
    L.srt_debug_fail_alloc(0)
    try:
        with pytest.raises(srt.SrtError) as ei:
            srt.Fields(phi, b)
        assert ei.value.code == SRT_ERR_OUT_OF_MEMORY
        # the failure was taken: the next handle is created normally
        with srt.Fields(phi, b) as f:
            maps, _ = f.forward(2, 8, precision="fp64")
        assert np.all(np.isfinite(maps))
    finally:
        L.srt_debug_fail_alloc(-1)
