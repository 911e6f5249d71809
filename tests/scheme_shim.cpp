// Host build of the MIXED form's cell lookup (snapshot-raytracer_gb300/csrc/srt_scheme.cuh,
// locate_mixed) for tests/test_locate_mixed.py.
#include "srt_scheme.cuh"
extern "C" {
void locate(float th, float lo, int n, int* cc, float* tc, int* cs, float* ts, float* df) {
  srt::locate_mixed(th, lo, n, 1.0f / (float)n, *cc, *tc, *cs, *ts, *df);
}
}
