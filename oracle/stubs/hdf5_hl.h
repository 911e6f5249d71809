/* Empty stand-in for hdf5_hl.h (the reference includes it but calls nothing from it). */
#pragma once
#include "hdf5.h"
