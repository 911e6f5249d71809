"""Regenerate tests/golden/golden_maps.npz from the reference's OWN host code.

The reference (snapshot-raytracer.cu) has no tests or known-answer vectors, so
the golden vectors are produced here by running its tracing functions
(compiled from the reference sources by oracle/build_ref.sh into
oracle/_ref/libsrt_ref.so) on bit-reproducible integer-noise fields
(srt_fields.int_noise_fields: exact float32 values on any platform). Only the
maps are stored; the fields are regenerated from the recorded seeds.

Needs the reference sources (this script runs only where they exist):
    python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "snapshot-raytracer_gb300"))
sys.path.insert(0, ROOT)

import srt_fields  # noqa: E402
from oracle import oracle  # noqa: E402

# name: (extents (n0, n1, n2), seed, nside, n_steps, batch or None, zero fields)
CASES = {
    "cube16_ns2_s12": ((16, 16, 16), 1, 2, 12, None, False),
    "cube32_ns4_s24": ((32, 32, 32), 2, 4, 24, None, False),
    "cube24_ns3_s20": ((24, 24, 24), 3, 3, 20, None, False),
    "wrap16_ns2_s40": ((16, 16, 16), 4, 2, 40, None, False),
    "batch5_cube32_ns4_s16": ((32, 32, 32), 5, 4, 16, 5, False),
    "noncubic_16x20x24_ns2_s14": ((16, 20, 24), 6, 2, 14, None, False),
    "zero16_ns2_s10": ((16, 16, 16), 7, 2, 10, None, True),
}

# interpolation points: (case, field, x, y, z) — field 0..2 = B components, 3 = phi
INTERP_POINTS = [("cube16_ns2_s12", f, x, y, z) for f in range(4)
                 for (x, y, z) in ((3.25, 7.5, 9.125), (0.0, 15.999, 8.5), (-2.75, 20.5, 4.0), (8.0, 8.0, 8.0))]


def fields_of(case):
    ext, seed, _, _, _, zero = CASES[case]
    phi, b = srt_fields.int_noise_fields(ext, seed)
    if zero:
        phi, b = np.zeros_like(phi), np.zeros_like(b)
    return phi, b


def full_maps(case, part, begin):
    _, _, nside, _, _, _ = CASES[case]
    full = np.zeros((6, 12 * nside * nside), np.float32)
    full[:, begin:begin + part.shape[1]] = part
    return full


def main():
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref/libsrt_ref.so is missing: run oracle/build_ref.sh first")
    out, meta = {}, {"generator": "srt_fields.int_noise_fields", "source": "reference host code via oracle/_ref",
                     "cases": {}, "interp_points": INTERP_POINTS}
    for name, (ext, seed, nside, steps, batch, zero) in CASES.items():
        phi, b = fields_of(name)
        begin, count = (0, 12 * nside * nside) if batch is None else (batch * nside * nside, nside * nside)
        part = oracle.ref_trace(phi, b, nside, steps, begin, count)
        out[name] = full_maps(name, part, begin)
        meta["cases"][name] = {"extents": ext, "seed": seed, "nside": nside, "n_steps": steps, "batch": batch,
                               "zero_fields": zero}
    vals = []
    for case, f, x, y, z in INTERP_POINTS:
        phi, b = fields_of(case)
        vals.append(oracle.ref_interp(phi, b, f, x, y, z))
    out["interp"] = np.array(vals, np.float64)
    np.savez_compressed(os.path.join(HERE, "golden_maps.npz"), **out)
    with open(os.path.join(HERE, "golden_cases.json"), "w") as fh:
        json.dump(meta, fh, indent=1)
    print("wrote", len(CASES), "cases")


if __name__ == "__main__":
    main()
