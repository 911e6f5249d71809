// srt_adjoint.cu — reverse-mode (vjp) kernels of the tracer (placeholder).
#include "srt_internal.h"
