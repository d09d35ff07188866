// Headless stand-in for the reference's libs/common/include/common/umbrella.h (see macros.h in this
// directory). Pulls in the configuration constants and the CUDACHECK macro; <initializer_list> is needed by
// the reference's graph helpers (cuda-internal.cuh:60-81) and is not included by anything else there.
#pragma once
#include <initializer_list>
#include <stdint.h>

#include "constants.h"
#include "macros.h"
