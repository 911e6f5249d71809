// srt_io.cpp — host file formats (placeholder until the HDF5 / FITS codecs land).
#include "srt.h"
#include "srt_internal.h"
extern "C" {
int srt_h5_read_scalar(const char*, const char*, float**, int64_t*, int*) { return srt::set_error(SRT_ERR_UNSUPPORTED, "not built"); }
int srt_h5_read_vector3(const char*, const char*, float**, int64_t*) { return srt::set_error(SRT_ERR_UNSUPPORTED, "not built"); }
int srt_h5_write(const char*, const char*, const float*, const int64_t*, int, int) { return srt::set_error(SRT_ERR_UNSUPPORTED, "not built"); }
int srt_fits_write_map(const char*, const float*, int64_t, int, const char*, int) { return srt::set_error(SRT_ERR_UNSUPPORTED, "not built"); }
int srt_fits_read_map(const char*, float**, int64_t*, int64_t*, int*) { return srt::set_error(SRT_ERR_UNSUPPORTED, "not built"); }
}
