"""Parity at the small named configuration, on every pixel of the batch: a
periodic 128^3 grid with the observer at the box centre, phi a Gaussian
random field with P(k) ~ k^-3 (0 < k <= k_Nyquist, zero mode removed) at
real-space rms 1e-5 and B a transverse Gaussian field of the same spectrum at
rms 1e-7 (numpy generator, seed 128), traced at nside 32 for 64 steps, batch 0
(RING pixels [0, 1024)), as the reference's CLI runs it
(snapshot-raytracer.cu:708-717, kernel launch :897-901).

Checked against the FP64 host oracle on all 1024 pixels: the FP64 GPU form,
the MIXED form and the REF16 form (the reference's own arithmetic); and the
reference's own GPU build (its unmodified raytracing_kernel) against the
oracle, against this library's FP64 form and against its REF16 form. The
bounds are stated per comparison (relative to each map's rms signal, one
float32 ulp of resolution not counted; map_errors in oracle/oracle.py); they
sit a few times above the errors measured on a GB300."""
import numpy as np
import pytest

import srt_fields
from conftest import map_errors

pytestmark = pytest.mark.gpu

N, NSIDE, STEPS, BATCH, SEED = 128, 32, 64, 0, 128
BEGIN, COUNT = BATCH * NSIDE * NSIDE, NSIDE * NSIDE

# (rms, max) bounds per comparison, a few times the errors measured on a GB300
# (in brackets: the largest rms and max over the six maps)
BOUNDS = {
    "fp64_vs_oracle": (1e-8, 1e-7),      # the same FP64 scheme: identical floats [0, 0]
    "mixed_vs_oracle": (5e-7, 3e-6),     # [1.3e-7, 7.5e-7]; the MIXED target is rms <= 1e-5
    "ref16_vs_oracle": (2e-5, 1e-4),     # the reference's FP16 B planes, FP32 cell offsets [5.3e-6, 2.8e-5]
    "refgpu_vs_oracle": (2e-5, 4e-4),    # [5.3e-6, 1.1e-4]
    "refgpu_vs_fp64": (2e-5, 4e-4),      # [5.3e-6, 1.1e-4]
    "refgpu_vs_ref16": (1.5e-5, 4e-4),   # same arithmetic, --use_fast_math rounding order [3.5e-6, 1.1e-4]
}


@pytest.fixture(scope="module")
def config1(srt, orc):
    phi, b = srt_fields.gaussian_fields_np(N, seed=SEED)
    want = orc.trace(phi, b, NSIDE, STEPS, BEGIN, COUNT, mode="fp64")
    got = {}
    with srt.Fields(phi, b) as f:
        for mode in ("fp64", "mixed", "ref16"):
            got[mode], _ = f.forward(NSIDE, STEPS, BEGIN, COUNT, precision=mode)
    ref = None
    if orc.ref_gpu_available():
        import torch

        ref_t, _ = orc.ref_gpu_trace(torch.from_numpy(phi).cuda(), torch.from_numpy(b).cuda(), NSIDE, STEPS, BEGIN,
                                     COUNT)
        ref = ref_t.cpu().numpy()
    return want, got, ref


def _check(name, a, b):
    rms_b, max_b = BOUNDS[name]
    errs = map_errors(a, b)
    for m, (rms, mx) in enumerate(errs):
        assert rms <= rms_b and mx <= max_b, "%s, map %d: rms %.3g (bound %.1g), max %.3g (bound %.1g)" % (
            name, m, rms, rms_b, mx, max_b)
    return errs


@pytest.mark.parametrize("mode", ["fp64", "mixed", "ref16"])
def test_config1_forms_vs_fp64_oracle(config1, mode):
    want, got, _ = config1
    assert got[mode].shape == (6, COUNT) and np.all(np.isfinite(got[mode]))
    _check("%s_vs_oracle" % mode, got[mode], want)


def test_config1_reference_build(config1):
    want, got, ref = config1
    if ref is None:
        pytest.skip("reference GPU build not available")
    assert np.all(np.isfinite(ref))
    _check("refgpu_vs_oracle", ref, want)
    _check("refgpu_vs_fp64", ref, got["fp64"])
    _check("refgpu_vs_ref16", ref, got["ref16"])
